"""Generates tests/golden/relief_samples.npz: the reference's relief and
colour sampling and its key-light shadow march (shaders/render.wgsl,
translated by oracle/wgsl_ref and evaluated in FP64 by
oracle/_ref/librenderref.so) on a small seeded film.

Runs where the reference checkout exists (REFERENCE, else where
oracle/wgsl_ref/build_ref.py's reference_root finds it).
Usage: python tests/golden/make_relief.py
"""
import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "paint-sim-3d_gb300"))


def film_planes(w, h, seed):
    """Blobs with sharp rims (the colour sharpening's edge path), a weave
    relief and a colour field, all as the film stores them (f32 h, m; f16 colour)."""
    from canvaz_film import synth
    cv = synth.blob_canvas(w, h, seed, n_blobs=6, sigma=(2, 6), per_cell_n=False, tables="reference")
    hp = np.asarray(cv.planes["h"], np.float32).reshape(-1)
    rng = np.random.Generator(np.random.PCG64(seed))
    hp = np.where(rng.random(hp.size) < 0.1, 0.0, hp).astype(np.float32)  # holes: wet / dry edges
    mp = (np.asarray(cv.planes["m"], np.float32).reshape(-1) + rng.uniform(0, 2e-5, hp.size)).astype(np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    col = np.stack([0.5 + 0.4 * np.sin(xx / 5.0), 0.5 + 0.4 * np.cos(yy / 7.0), rng.uniform(0.05, 0.9, (h, w)),
                    rng.uniform(0.06, 0.85, (h, w))], -1).astype(np.float16)
    return cv.settings["width_m"], cv.settings["height_m"], hp, mp, col.reshape(-1, 4)


def main():
    sys.path.insert(0, str(ROOT / "oracle" / "wgsl_ref"))
    import build_ref
    ref = str(build_ref.reference_root())
    subprocess.run([sys.executable, str(ROOT / "oracle" / "wgsl_ref" / "build_ref.py"), ref], check=True)
    L = C.CDLL(str(ROOT / "oracle" / "_ref" / "librenderref.so"))
    fp = C.POINTER(C.c_float)
    L.wgrr_set.argtypes = [C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_float, fp, fp, fp]
    L.wgrr_sample.argtypes = [C.POINTER(C.c_double), C.c_uint32, C.POINTER(C.c_double)]
    w, h = 40, 32
    wm, hm, hp, mp, col = film_planes(w, h, 7)
    dx = np.float32(wm) / np.float32(w)
    colf = np.ascontiguousarray(col.astype(np.float32))
    L.wgrr_set(w, h, wm, hm, dx, hp.ctypes.data_as(fp), mp.ctypes.data_as(fp), colf.ctypes.data_as(fp))
    rng = np.random.Generator(np.random.PCG64(11))
    pts = [rng.uniform(-0.05, 1.05, (3000, 2)) * np.array([wm, hm])]  # inside and around the canvas
    # near every cell centre and near every cell edge; exactly at a centre the
    # sample grid's floor() sits on its discontinuity, where an f32 and an
    # FP64 evaluation of the same shader pick different cells
    cx, cy = np.meshgrid((np.arange(w) + 0.5) * dx, (np.arange(h) + 0.5) * dx)
    pts.append(np.stack([cx.ravel() + 0.013 * dx, cy.ravel() + 0.021 * dx], 1))
    pts.append(np.stack([cx.ravel() + 0.5 * dx, cy.ravel() + 0.25 * dx], 1))
    pts = np.concatenate(pts).astype(np.float32)
    out = np.zeros((len(pts), 8), np.float64)
    p64 = np.ascontiguousarray(pts.astype(np.float64))
    L.wgrr_sample(p64.ctypes.data_as(C.POINTER(C.c_double)), len(pts), out.ctypes.data_as(C.POINTER(C.c_double)))
    # the key-light shadow march (shadow_at) from the bilinear surface height
    # of each point, for a high, a low and a grazing light; the march stops at the top of
    # the relief volume (cam.canvas.w = max(h + m) + 0.5 mm)
    L.wgrr_set_top.argtypes = [C.c_float]
    L.wgrr_shadow.argtypes = [C.POINTER(C.c_double), C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    top = np.float32(float(np.max(hp + mp)) + 0.5e-3)
    L.wgrr_set_top(top)
    sp = np.zeros((len(pts), 3), np.float64)
    sp[:, :2] = pts
    lights = np.array([[0.6, 0.2, 0.5], [-0.3, -0.7, 0.25], [0.9, 0.3, 0.08]], np.float32)
    lights = (lights / np.linalg.norm(lights, axis=1, keepdims=True)).astype(np.float32)
    sh_out = []
    for li in lights:
        l64 = np.ascontiguousarray(li.astype(np.float64))
        o = np.zeros((len(pts), 2), np.float64)
        L.wgrr_shadow(sp.ctypes.data_as(C.POINTER(C.c_double)), len(pts), l64.ctypes.data_as(C.POINTER(C.c_double)),
                      o.ctypes.data_as(C.POINTER(C.c_double)))
        sp[:, 2] = o[:, 0].astype(np.float32)  # z0 = the surface height under the point
        L.wgrr_shadow(sp.ctypes.data_as(C.POINTER(C.c_double)), len(pts), l64.ctypes.data_as(C.POINTER(C.c_double)),
                      o.ctypes.data_as(C.POINTER(C.c_double)))
        sh_out.append(o)
    np.savez_compressed(HERE / "relief_samples.npz", w=w, h=h, width_m=wm, height_m=hm, h_plane=hp, m_plane=mp,
                        color_f16=col.view(np.uint16), points=pts, out=out, shadow_z0=sp[:, 2].astype(np.float32),
                        shadow_top=top, shadow_lights=lights, shadow_out=np.stack(sh_out))
    print("shadow samples: %d per light, in shadow (< 1): %s" % (
        len(pts), [int((o[:, 1] < 1).sum()) for o in sh_out]))
    print("relief_samples: %d points, edge-blended colour at %d" % (
        len(pts), int((np.abs(out[:, 3:7]).sum(1) > 0).sum())))


if __name__ == "__main__":
    main()
