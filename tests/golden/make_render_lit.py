"""Generates tests/golden/render_lit.npz: the reference renderer's whole
fragment shader (shaders/render.wgsl fs and lit: the ray march over the
relief, the tool micro-relief of the detail texture, the canvas weave, the
beauty-mode colour, shadow, ambient occlusion, environment, softbox and GGX
lobes, tonemap and sRGB), translated by oracle/wgsl_ref and evaluated in f32
with one rounding per operation, as the shader computes, by
oracle/_ref/librenderfsref.so, for the pixels of small images of a seeded
film seen by four cameras: top-down orthographic, oblique perspective, the
perspective camera with a thin lens, and the beauty mode.

Runs where the reference checkout exists (REFERENCE, else where
oracle/wgsl_ref/build_ref.py's reference_root finds it).
Usage: python tests/golden/make_render_lit.py
"""
import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "paint-sim-3d_gb300"))

IMG_W, IMG_H = 48, 36


def film_planes(w, h, seed):
    """Blobs with holes (wet / dry edges) over a weave relief, a colour field
    as the film stores it (rgba16f: rgb and roughness), and a detail texture
    with brush, knife and roller strokes at random turns, cure fractions,
    yield stresses and the thickness of the paint (rgba16f)."""
    from canvaz_film import synth
    cv = synth.blob_canvas(w, h, seed, n_blobs=6, sigma=(2, 6), per_cell_n=False, tables="reference")
    rng = np.random.Generator(np.random.PCG64(seed))
    hp = np.asarray(cv.planes["h"], np.float32).reshape(-1)
    hp = np.where(rng.random(hp.size) < 0.08, 0.0, hp).astype(np.float32)
    mp = (np.asarray(cv.planes["m"], np.float32).reshape(-1) + rng.uniform(0, 2e-5, hp.size)).astype(np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    col = np.stack([0.5 + 0.4 * np.sin(xx / 5.0), 0.5 + 0.4 * np.cos(yy / 7.0), rng.uniform(0.05, 0.9, (h, w)),
                    rng.uniform(0.06, 0.85, (h, w))], -1).astype(np.float16).reshape(-1, 4)
    method = rng.choice([0.0, 4.0, 5.0, 6.0], size=hp.size, p=[0.25, 0.35, 0.25, 0.15])
    turn = rng.uniform(0, 1, hp.size)
    thick = hp + np.maximum(mp - 60e-6, 0.0)
    det = np.stack([method + turn, rng.uniform(0, 1, hp.size), rng.uniform(0, 40, hp.size), thick], -1)
    det = det.astype(np.float16).reshape(-1, 4)
    tw, th = (w + 15) // 16, (h + 15) // 16
    flags = (rng.random(tw * th) < 0.6).astype(np.uint32)
    return cv.settings["width_m"], cv.settings["height_m"], hp, mp, col, det, flags


def look_at_rh(eye, target, up):
    f = target - eye
    f = f / np.linalg.norm(f)
    s = np.cross(f, up)
    s = s / np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.identity(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def perspective_rh_zo(fov, aspect, near, far):
    hh = 1.0 / np.tan(0.5 * fov)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = hh / aspect, hh
    m[2, 2], m[2, 3] = far / (near - far), near * far / (near - far)
    m[3, 2] = -1.0
    return m


def cam_words(width_m, height_m, dx, top, w, h, kind):
    """The Cam uniform (76 words) the renderer would write for this camera."""
    target = np.array([0.5 * width_m, 0.5 * height_m, 0.0])
    yaw, pitch, dist = (0.6, 0.85, 1.6 * width_m) if kind != "beauty" else (-1.1, 0.95, 1.3 * width_m)
    eye = target + dist * np.array([np.cos(pitch) * np.cos(yaw), np.cos(pitch) * np.sin(yaw), np.sin(pitch)])
    vp = perspective_rh_zo(0.8, IMG_W / IMG_H, 0.01, 20.0) @ look_at_rh(eye, target, np.array([0.0, 0.0, 1.0]))
    inv = np.linalg.inv(vp)
    light = np.array([0.45, -0.3, 0.84])
    light = light / np.linalg.norm(light)
    words = []
    words += list(inv.T.reshape(-1))            # columns
    words += [eye[0], eye[1], eye[2], 0.0]
    words += [width_m, height_m, dx, top]
    words += [light[0], light[1], light[2], 3.0]
    size = np.array([w, h, 0, 0], np.uint32).view(np.float32)  # u32 words, set below by bit pattern
    words += [None] * 4
    words += [0.55, 0.62, 0.7, 1.0]             # sky
    words += [0.2, 0.18, 0.16, 1.0]             # ground
    words += list(vp.T.reshape(-1))
    jitter = [0.0, 0.0, 1.0 if kind == "beauty" else 0.0, 0.0]
    words += jitter
    words += [1.0 if kind == "ortho" else 0.0, np.tan(np.radians(35.0)), 0.0, 0.0]  # ortho.y: tan(contact angle)
    r = np.array([np.sin(yaw), -np.cos(yaw), 0.0])
    u = np.cross(r, (target - eye) / dist)
    words += [r[0], r[1], r[2], 0.0]            # basis_r
    words += [u[0], u[1], u[2], 0.0]            # basis_u
    words += [0.004 * width_m, -0.003 * width_m, dist, 1.0] if kind == "lens" else [0.0] * 4
    out = np.zeros(76, np.float32)
    for k, v in enumerate(words):
        if v is not None:
            out[k] = np.float32(v)
    out[28:32] = size
    return out


def pixel_ndc():
    """The interpolated ndc of each pixel centre of an IMG_W x IMG_H target."""
    px, py = np.meshgrid(np.arange(IMG_W) + 0.5, np.arange(IMG_H) + 0.5)
    return np.stack([2.0 * px / IMG_W - 1.0, 1.0 - 2.0 * py / IMG_H], -1).reshape(-1, 2).astype(np.float32)


def main():
    sys.path.insert(0, str(ROOT / "oracle" / "wgsl_ref"))
    import build_ref
    ref = str(build_ref.reference_root())
    subprocess.run([sys.executable, str(ROOT / "oracle" / "wgsl_ref" / "build_ref.py"), ref], check=True)
    L = C.CDLL(str(ROOT / "oracle" / "_ref" / "librenderfsref.so"))
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
    L.wgrf_set.argtypes = [fp, C.c_uint32, C.c_uint32, fp, fp, fp, fp, C.POINTER(C.c_uint32)]
    L.wgrf_fs.argtypes = [dp, C.c_uint32, dp]
    w, h = 40, 32
    wm, hm, hp, mp, col, det, flags = film_planes(w, h, 5)
    dx = np.float32(wm) / np.float32(w)
    top = np.float32(float(np.max(hp + mp)) + 0.5e-3)
    colf = np.ascontiguousarray(col.astype(np.float32))
    detf = np.ascontiguousarray(det.astype(np.float32))
    ndc = pixel_ndc()
    kinds = ["ortho", "persp", "lens", "beauty"]
    cams, outs = [], []
    for kind in kinds:
        cw = cam_words(wm, hm, dx, top, w, h, kind)
        L.wgrf_set(cw.ctypes.data_as(fp), w, h, hp.ctypes.data_as(fp), mp.ctypes.data_as(fp), colf.ctypes.data_as(fp),
                   detf.ctypes.data_as(fp), flags.ctypes.data_as(C.POINTER(C.c_uint32)))
        o = np.zeros((len(ndc), 4), np.float64)
        n64 = np.ascontiguousarray(ndc.astype(np.float64))
        L.wgrf_fs(n64.ctypes.data_as(dp), len(ndc), o.ctypes.data_as(dp))
        cams.append(cw)
        outs.append(o)
        print("%-6s rgb mean %s, min %s, max %s" % (kind, o[:, :3].mean(0).round(3), o[:, :3].min(0).round(3),
                                                   o[:, :3].max(0).round(3)))
    np.savez_compressed(HERE / "render_lit.npz", w=w, h=h, width_m=wm, height_m=hm, h_plane=hp, m_plane=mp,
                        color_f16=col.view(np.uint16), detail_f16=det.view(np.uint16), tile_flags=flags,
                        img_w=IMG_W, img_h=IMG_H, ndc=ndc, kinds=np.array(kinds), cams=np.stack(cams),
                        out=np.stack(outs))


if __name__ == "__main__":
    main()
