"""Generates tests/golden/resolve_samples.npz: the reference's display
fragment shader (shaders/resolve.wgsl fs, translated by oracle/wgsl_ref and
evaluated in f32 by oracle/_ref/libresolveref.so) over a small seeded HDR
image, for five settings of its Res uniform (AgX / ACES, exposure, bloom,
sharpen, vignette, grain).

Runs where the reference checkout exists (REFERENCE, else where
oracle/wgsl_ref/build_ref.py's reference_root finds it).
Usage: python tests/golden/make_resolve.py
"""
import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "resolve_samples.npz"
W, H = 48, 40
# (scale, exposure_ev, bloom, grain, vignette, sharpen, agx)
CASES = [(1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1), (1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0),
         (3.0, 0.0, 0.8, 0.0, 0.0, 0.0, 1), (1.0, 0.0, 0.0, 0.3, 0.4, 0.6, 1),
         (4.0, 0.0, 0.5, 0.0, 0.0, 0.3, 0)]


def image(seed=3):
    """Linear RGB with smooth ramps, dark corners and a few bright spots (so
    the bloom's threshold at luminance 1.6 is crossed), stored as f16."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    r = 0.05 + 0.9 * xx / W
    g = 0.02 + 0.7 * (1 + np.sin(yy / 6.0)) / 2
    b = 0.1 + 0.6 * rng.random((H, W))
    img = np.stack([r, g, b, np.full((H, W), 0.35)], -1)
    for _ in range(5):
        cx, cy = rng.integers(4, W - 4), rng.integers(4, H - 4)
        img[cy - 1:cy + 2, cx - 1:cx + 2, :3] = rng.uniform(2.0, 6.0, 3)
    img[:6, :6, :3] = 0.001
    return img.astype(np.float16)


def res12(case):
    scale, ev, bloom, grain, vig, sharpen, agx = case
    return np.array([scale, ev, bloom, grain, vig, W, H, float(agx), sharpen, 0, 0, 0], np.float32)


def main():
    sys.path.insert(0, str(ROOT / "oracle" / "wgsl_ref"))
    import build_ref
    ref = str(build_ref.reference_root())
    subprocess.run([sys.executable, str(ROOT / "oracle" / "wgsl_ref" / "build_ref.py"), ref], check=True)
    L = C.CDLL(str(ROOT / "oracle" / "_ref" / "libresolveref.so"))
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
    L.wgres_run.argtypes = [C.c_uint32, C.c_uint32, fp, fp, dp]
    img = image()
    src = np.ascontiguousarray(img.astype(np.float32).reshape(-1))
    outs, params = [], []
    for case in CASES:
        r = res12(case)
        out = np.zeros(W * H * 4, np.float64)
        L.wgres_run(W, H, src.ctypes.data_as(fp), r.ctypes.data_as(fp), out.ctypes.data_as(dp))
        outs.append(out.reshape(H, W, 4))
        params.append(np.array(case, np.float64))
    np.savez_compressed(OUT, w=W, h=H, image_f16=img.view(np.uint16), cases=np.array(params), out=np.array(outs))
    print("wrote", OUT, np.array(outs).shape)


if __name__ == "__main__":
    main()
