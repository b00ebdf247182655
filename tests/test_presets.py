"""The reference's built-in scenes (pg3render_gb300.presets): every -s id builds, and the scenes
carry the reference's lights.
Their renders are checked against the reference's own scene construction by the preset_*
golden fixtures (tests/test_oracle.py, tests/test_gpu_parity.py)."""
import math

import numpy as np
import pytest

from pg3render_gb300 import presets as PR
from pg3render_gb300 import scene as S


def test_every_scene_id_builds():
    for sid in range(len(PR.SCENE_CONFIGS)):
        sc = PR.reference_scene(sid, 8, 8)
        assert len(sc.materials) == 13 and sc.num_lights >= 1
        mask = PR.SCENE_CONFIGS[sid]
        assert (len(sc.point_lights) == 1) == bool(mask & PR.LIGHT_POINT)
        assert sc.has_background == bool(mask & PR.LIGHT_ENV)
        text = sc.to_text(max_path_length=8)
        assert text.startswith("# reference_scene_%d" % sid)
        assert ("\nsra " in text) == (sid == 27)   # the SRA layered sphere


def test_area_lights_emit_25_watts():
    for sid in (2, 4):   # ceiling light, light box
        sc = PR.reference_scene(sid, 8, 8)
        assert len(sc.area_lights) == 2
        flux = 0.0
        for t, L in sc.area_lights:
            p0, p1, p2 = (np.asarray(v) for v in sc.triangles[t][:3])
            area = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0))
            flux += math.pi * area * L[0]    # radiance = flux / (pi * area), src/lights.hxx:107-112
            n = np.cross(p1 - p0, p2 - p0)
            assert n[2] < 0                  # emits downwards
        assert abs(flux - 25.0) < 1e-4


def test_environment_types():
    sc = PR.reference_scene(6, 8, 8)
    assert sc.background_const == (135 / 255.0, 206 / 255.0, 250 / 255.0)
    sc = PR.reference_scene(6, 8, 8, env_type=PR.EM_CONST_SRGB_WHITE)
    assert sc.background_const == (0.87, 0.87, 0.87)
    with pytest.raises(ValueError):
        PR.reference_scene(6, 8, 8, env_type=PR.EM_IMG_PISA)     # an EXR probe: texels needed
    em = S.synthetic_sky(32, 16, seed=1)
    sc = PR.reference_scene(6, 8, 8, env_type=PR.EM_IMG_PISA, env_map=em)
    assert sc.env_map.shape == (16, 32, 3)
    with pytest.raises(ValueError):
        PR.reference_scene(39, 8, 8)
