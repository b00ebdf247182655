"""Image files (pg3gpu_write_image / pg3gpu_save_image): the library's BMP and Radiance HDR
writers against the files the reference's own Framebuffer::SaveBMP and SaveHDR wrote from the
same framebuffer (tests/golden/image_writer.npz, made by tests/golden/make_golden.py). CPU only:
the writers need no GPU."""
import os

import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture():
    z = np.load(os.path.join(HERE, "golden", "image_writer.npz"))
    return z["framebuffer"], z["bmp"].tobytes(), z["hdr"].tobytes()


def test_bmp_matches_the_reference_writer(tmp_path):
    fb, ref, _ = _fixture()
    p = str(tmp_path / "img.bmp")
    P.write_image(fb, p, gamma=2.2)
    mine = open(p, "rb").read()
    h, w = fb.shape[:2]
    assert len(mine) == 54 + w * h * 3 and mine[:2] == b"BM"
    # the reference's header stores width*width*3 as the pixel bytes of the file size; every
    # other header field and every pixel byte must agree (rows need no padding at width 16)
    assert mine[6:54] == ref[6:54]
    assert mine[54:] == ref[54:]
    assert int.from_bytes(mine[2:6], "little") == len(mine)


def test_hdr_matches_the_reference_writer(tmp_path):
    fb, _, ref = _fixture()
    p = str(tmp_path / "img.hdr")
    P.write_image(fb, p)
    mine = open(p, "rb").read()
    h, w = fb.shape[:2]
    res = b"-Y %d +X %d\n" % (h, w)
    assert mine.startswith(b"#?RADIANCE\n") and b"FORMAT=32-bit_rle_rgbe\n\n" in mine and res in mine
    assert mine[mine.index(res) + len(res):] == ref[ref.index(res) + len(res):]


def test_bmp_rows_are_padded_and_bottom_up(tmp_path):
    img = np.zeros((2, 3, 3))
    img[0, 0] = (1.0, 0.0, 0.0)        # top-left red
    img[1, 2] = (0.0, 0.0, 1.0)        # bottom-right blue
    p = str(tmp_path / "pad.bmp")
    P.write_image(img, p, gamma=1.0)
    b = open(p, "rb").read()
    assert len(b) == 54 + 2 * 12       # 9 bytes per row padded to 12
    bottom, top = b[54:66], b[66:78]
    assert bottom[6:9] == bytes([255, 0, 0]) and top[0:3] == bytes([0, 0, 255])   # BGR


def test_image_argument_errors(tmp_path):
    L = _lib.load()
    assert L.pg3gpu_write_image(None, 1, 1, b"x.bmp", 2.2) == _lib.ERR_INVALID_ARGUMENT
    img = np.ones((1, 1, 3))
    with pytest.raises(_lib.Pg3Error):
        P.write_image(img, str(tmp_path / "x.bmp"), gamma=0.0)
    with pytest.raises(_lib.Pg3Error):
        P.write_image(img, str(tmp_path / "no_such_dir" / "x.hdr"))
    assert L.pg3gpu_save_image(None, b"x.bmp", 2.2) == _lib.ERR_INVALID_ARGUMENT
