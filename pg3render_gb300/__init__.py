"""GB300 (sm_103a) path-tracing hot path of PG3Render behind the reference's
renderer interface. The compute path is the CUDA library built from csrc/
(``build.build()``); this package only holds the scene builders and a thin
host-side mirror of the renderer interface over the library's C ABI."""
from . import diff, presets, scene  # noqa: F401
from .renderer import Config, GpuBatch, GpuPathTracer, Pg3Error, render, steerable_file_name, write_image  # noqa: F401

__all__ = ["diff", "presets", "scene", "Config", "GpuBatch", "GpuPathTracer", "Pg3Error", "render", "steerable_file_name",
           "write_image"]
