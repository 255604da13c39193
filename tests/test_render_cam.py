"""The renderer's camera uniform on the host (CPU): cf_render_cam has the
layout of render.wgsl's Cam (76 words), and canvaz_film.camera fills it as
the reference's Renderer::uniform does (vp and its inverse, the canvas, the
film size as u32 words, the modes)."""
import ctypes as C

import numpy as np

from canvaz_film import camera, capi


def test_layout_is_the_shader_uniform():
    assert C.sizeof(capi.RenderCam) == 76 * 4
    offs = {name: getattr(capi.RenderCam, name).offset // 4 for name, _ in capi.RenderCam._fields_}
    assert offs == {"inv_vp": 0, "eye": 16, "canvas": 20, "light": 24, "size": 28, "sky": 32, "ground": 36,
                    "vp": 40, "jitter": 56, "ortho": 60, "basis_r": 64, "basis_u": 68, "lens": 72}


def test_words_round_trip():
    w = np.arange(76, dtype=np.float32)
    w[28:32] = np.array([40, 32, 0, 0], np.uint32).view(np.float32)
    c = capi.RenderCam.from_words(w)
    assert list(c.size) == [40, 32, 0, 0]
    assert np.array_equal(np.frombuffer(bytes(c), np.float32), w)


def test_orbit_camera():
    c = camera.render_cam(64, 48, 0.032, 0.024, 3e-3, yaw=0.4, pitch=0.9, aspect=4 / 3, beauty=True,
                          lens=(1e-4, 0.0, 0.05))
    vp = np.array(c.vp, np.float64).reshape(4, 4).T
    inv = np.array(c.inv_vp, np.float64).reshape(4, 4).T
    assert np.allclose(inv @ vp, np.identity(4), atol=1e-4)
    # the canvas centre projects inside the view, in front of the camera
    p = vp @ np.array([0.016, 0.012, 0.0, 1.0])
    assert p[3] > 0 and np.all(np.abs(p[:2] / p[3]) < 1.0) and 0.0 <= p[2] / p[3] <= 1.0
    assert list(c.size) == [64, 48, 0, 0]
    assert c.jitter[2] == 1.0 and c.lens[3] == 1.0 and c.ortho[0] == 0.0
    assert np.isclose(c.canvas[2], 0.032 / 64) and np.isclose(c.canvas[3], 3e-3)
    eye = np.array(c.eye[:3])
    assert eye[2] > 0  # above the canvas
