"""Inverse rendering with the path-replay adjoint (no counterpart in the reference).

Recovers the environment map and six material parameters of the environment-lit box (the
albedos of its four Lambert materials and the roughnesses of two GGX spheres) from a target
image rendered with hidden, seeded values. Every iteration renders the current parameters
(forward + adjoint through the library's CUDA kernels), takes an L2 image loss and an Adam
step; the whole iteration -- parameter upload with the environment-map CDF rebuilt on the
device, forward, loss, adjoint, optimiser, and the advance of the sample offset so that each
replay draws new samples -- is one captured CUDA graph. Texels are optimised in log space.

One view of the box does not determine a sky: albedo times illumination is a scale ambiguity,
and the map absorbs the render noise. ``optimize_env=False`` keeps the map at its hidden values
(the materials are then identifiable); ``env_smoothness`` adds a penalty on the squared
differences of neighbouring log texels, which keeps the recovered map from fitting noise.

The L2 loss of a noisy render is biased: E[(X - t)^2] = (E[X] - t)^2 + Var[X], and the variance
term pulls the parameters towards darker, less noisy renders (albedos come out low). With
``decorrelate`` every iteration renders a second, independent estimate for the residual and
back-propagates 2 (X_a - t) dX_b/dparameters, whose expectation is the gradient of
(E[X] - t)^2 alone (one forward pass more per iteration).
"""
import math
import time

import numpy as np

from . import _lib, diff, renderer
from . import scene as S


def _hidden_scene(side, em, seed):
    rng = np.random.default_rng(seed)
    sc = S.cornell_env_diff(side, side, em[0], em[1], em_seed=1000 + seed)
    lam = [i for i, m in enumerate(sc.materials) if m.kind == S.MAT_LAMBERT]
    ggx = [i for i, m in enumerate(sc.materials) if m.kind != S.MAT_LAMBERT][:2]
    for i in lam:
        sc.materials[i].albedo = tuple(float(x) for x in rng.uniform(0.1, 0.9, 3))
    for i in ggx:
        sc.materials[i].alpha = float(math.exp(rng.uniform(math.log(0.05), math.log(0.5))))
    return sc, lam, ggx


def run(steps=500, lr=1e-2, side=128, spp=16, target_spp=1024, em=(256, 128), seed=0, max_path_length=12,
        rr_min_path_length=4, eval_spp=256, optimize_env=True, env_smoothness=0.0, decorrelate=False, device=0):
    """Returns a dict: losses against the hidden-parameter render, parameter errors before and
    after, and the device time per iteration. With optimize_env False the map keeps its hidden
    values and only the materials are recovered; env_smoothness > 0 weights the penalty on
    neighbouring log-texel differences (added to the image loss)."""
    import torch
    torch.cuda.set_device(device)
    hidden, lam, ggx = _hidden_scene(side, em, seed)
    cfg = renderer.Config(scene=hidden, max_path_length=max_path_length, rr_min_path_length=rr_min_path_length,
                          em_sampler=_lib.EM_CDF, base_seed=seed + 1)
    dr = diff.DiffRenderer(cfg, device=device)
    try:
        m_true, e_true = dr.get_params()
        dr.use_torch_stream()
        target = torch.empty((side, side, 3), device="cuda")
        dr.forward_into(target, 1 << 20, target_spp)   # samples disjoint from the optimisation's

        # initial guess: grey albedos, roughness 0.2, a constant grey sky
        m0 = m_true.copy()
        for i in lam:
            m0[i, :3] = 0.5
        for i in ggx:
            m0[i, 3] = 0.2
        mask = torch.zeros((len(hidden.materials), 4), device="cuda")
        for i in lam:
            mask[i, :3] = 1
        for i in ggx:
            mask[i, 3] = 1
        mats = torch.tensor(m0, device="cuda", requires_grad=True)
        if optimize_env:
            theta = torch.full(e_true.shape, math.log(0.5), device="cuda", requires_grad=True)
        else:
            theta = torch.tensor(np.log(np.maximum(e_true, 1e-30)), device="cuda")
        mats.register_hook(lambda g: g * mask)
        opt = torch.optim.Adam([mats, theta] if optimize_env else [mats], lr=lr, capturable=True)
        offset = torch.zeros(1, dtype=torch.int32, device="cuda")
        dr.set_sample_offset(offset)

        def iteration():
            opt.zero_grad(set_to_none=False)
            env = torch.exp(theta) if optimize_env else None
            if decorrelate:
                with torch.no_grad():
                    dr.set_params(mats.detach(), None if env is None else env.detach())
                    img_a = torch.empty_like(target)
                    dr.forward_into(img_a, 1 << 22, spp)   # samples disjoint from img's
                img = diff.render(dr, mats, env, iteration=0, spp=spp)
                resid = img_a - target
                loss = (resid ** 2).mean()
                total = (2.0 * resid * img).mean()         # its gradient: 2 (X_a - t) dX_b / dtheta
            else:
                img = diff.render(dr, mats, env, iteration=0, spp=spp)
                loss = ((img - target) ** 2).mean()
                total = loss
            if optimize_env and env_smoothness > 0:
                dv = theta[1:] - theta[:-1]
                du = theta[:, 1:] - theta[:, :-1]
                total = total + env_smoothness * ((dv ** 2).mean() + (du ** 2).mean())
            total.backward()
            opt.step()
            with torch.no_grad():
                mats.copy_(torch.where(mask > 0, mats.clamp(0.001, 1.0), mats))
            offset.add_(spp)
            return loss

        def evaluate():
            with torch.no_grad():
                dr.set_sample_offset(None)
                dr.set_params(mats.detach(), torch.exp(theta).detach() if optimize_env else None)
                img = torch.empty_like(target)
                dr.forward_into(img, 1 << 24, eval_spp)
                dr.set_sample_offset(offset)
                m = mats.detach().cpu().numpy()
                e = torch.exp(theta).detach().cpu().numpy()
                return dict(loss=float(((img - target) ** 2).mean()),
                            albedo_mae=float(np.abs(m[lam, :3] - m_true[lam, :3]).mean()),
                            alpha_abs_err=float(np.abs(m[ggx, 3] - m_true[ggx, 3]).mean()),
                            env_rel_l1=float(np.abs(e - e_true).mean() / np.abs(e_true).mean()))

        before = evaluate()
        side_stream = torch.cuda.Stream()
        side_stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side_stream):
            for _ in range(3):
                iteration()
        torch.cuda.current_stream().wait_stream(side_stream)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            loss = iteration()
        losses = []
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        wall = time.perf_counter()
        t0.record()
        for k in range(steps - 3):
            graph.replay()
            if k % 50 == 0:
                losses.append(float(loss.detach()))
        t1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall
        after = evaluate()
        ms = t0.elapsed_time(t1) / max(1, steps - 3)
        return dict(steps=steps, side=side, spp=spp, target_spp=target_spp, env=list(e_true.shape),
                    optimize_env=optimize_env, env_smoothness=env_smoothness, decorrelate=decorrelate,
                    iteration_ms=ms, wall_s=wall, before=before, after=after, loss_trace=losses,
                    materials_true=m_true[lam + ggx].tolist(), materials_found=mats.detach().cpu().numpy()[lam + ggx].tolist())
    finally:
        dr.close()
