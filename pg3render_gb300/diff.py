"""Differentiable rendering over the C ABI (pg3gpu_set_params, pg3gpu_diff_forward,
pg3gpu_diff_adjoint) and its ``torch.autograd.Function`` binding.

The gradient is path-replay backpropagation computed by the library's CUDA kernels: the
forward keeps one radiance triple per path, the adjoint re-traces every path from its
random-number key. PyTorch only holds the device buffers and drives the optimiser.

Parameters: ``materials`` is (num_materials, 4) float32 -- albedo rgb of Lambert materials,
roughness alpha in column 3 of GGX materials; ``env`` is the environment map's
(height, width, 3) texels. No counterpart in the reference.
"""
import ctypes

import numpy as np

from . import _lib
from .renderer import GpuPathTracer, Pg3Error  # noqa: F401

PARAMS_DEVICE, PARAMS_KEEP_SAMPLING = 1, 2


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class DiffRenderer(GpuPathTracer):
    """A GpuPathTracer with the differentiable entry points."""

    @property
    def num_materials(self):
        return len(self.config.scene.materials)

    @property
    def env_shape(self):
        em = self.config.scene.env_map
        return None if em is None else tuple(em.shape)

    def use_torch_stream(self):
        import torch
        self.set_stream(torch.cuda.current_stream().cuda_stream)

    # -- host arrays ------------------------------------------------------------------------
    def get_params(self):
        m = np.zeros((self.num_materials, 4), np.float32)
        e = np.zeros(self.env_shape, np.float32) if self.env_shape else None
        _lib.check(self._L.pg3gpu_get_params(self._ctx, m.ctypes.data_as(ctypes.c_void_p),
                                             e.ctypes.data_as(ctypes.c_void_p) if e is not None else None), self._ctx)
        return m, e

    def set_params(self, materials=None, env=None, keep_sampling=False):
        """numpy arrays (host) or torch CUDA tensors (device, stream-ordered on torch's stream)."""
        flags = PARAMS_KEEP_SAMPLING if keep_sampling else 0
        if _is_torch(materials) or _is_torch(env):
            self.use_torch_stream()
            flags |= PARAMS_DEVICE
            args = (_dptr(_f32c(materials)), _dptr(_f32c(env)))
        else:
            m = None if materials is None else np.ascontiguousarray(materials, np.float32)
            e = None if env is None else np.ascontiguousarray(env, np.float32)
            args = (m.ctypes.data_as(ctypes.c_void_p) if m is not None else None,
                    e.ctypes.data_as(ctypes.c_void_p) if e is not None else None)
        _lib.check(self._L.pg3gpu_set_params(self._ctx, args[0], args[1], flags), self._ctx)

    def set_sample_offset(self, offset):
        """A one-element int32/uint32 CUDA tensor added to the sample indices of every
        differentiable launch (None: off); advancing it inside a captured graph renders new
        samples on every replay."""
        self._offset = offset
        _lib.check(self._L.pg3gpu_set_sample_offset(self._ctx, _dptr(offset)), self._ctx)

    # -- device tensors -----------------------------------------------------------------------
    def forward_into(self, image, iteration, spp):
        self.use_torch_stream()
        _lib.check(self._L.pg3gpu_diff_forward(self._ctx, iteration, spp, _dptr(image)), self._ctx)

    def adjoint_into(self, dloss_dimage, grad_materials, grad_env=None):
        self.use_torch_stream()
        _lib.check(self._L.pg3gpu_diff_adjoint(self._ctx, _dptr(_f32c(dloss_dimage)), _dptr(grad_materials),
                                               _dptr(grad_env)), self._ctx)


def _is_torch(x):
    return x is not None and type(x).__module__.startswith("torch")


def _f32c(t):
    if t is None:
        return None
    if not t.is_contiguous() or t.dtype != _torch().float32:
        raise ValueError("parameters must be contiguous float32 CUDA tensors")
    return t


def _torch():
    import torch
    return torch


def _make_function():
    torch = _torch()

    class RenderFunction(torch.autograd.Function):
        """image = render(materials, env); backward = the library's path-replay adjoint."""

        @staticmethod
        def forward(ctx, materials, env, renderer, iteration, spp, keep_sampling):
            renderer.set_params(materials.detach(), None if env is None else env.detach(), keep_sampling)
            img = torch.empty((renderer.height, renderer.width, 3), device=materials.device, dtype=torch.float32)
            renderer.forward_into(img, iteration, spp)
            ctx.renderer = renderer
            ctx.has_env = env is not None
            ctx.shapes = (materials.shape, None if env is None else env.shape)
            return img

        @staticmethod
        def backward(ctx, grad_img):
            r = ctx.renderer
            gm = torch.zeros(ctx.shapes[0], device=grad_img.device, dtype=torch.float32)
            ge = torch.zeros(ctx.shapes[1], device=grad_img.device, dtype=torch.float32) if ctx.has_env else None
            r.adjoint_into(grad_img.contiguous().float(), gm, ge)
            return gm, ge, None, None, None, None

    return RenderFunction


_fn = None


def render(renderer, materials, env=None, iteration=0, spp=16, keep_sampling=False):
    """Differentiable render: returns the (H, W, 3) mean image of samples iteration..+spp-1."""
    global _fn
    if _fn is None:
        _fn = _make_function()
    return _fn.apply(materials, env, renderer, iteration, spp, keep_sampling)
