"""CPU restatement of the resolve fragment (shaders/resolve.wgsl:23-121).

TEST INFRASTRUCTURE: the checker of the CUDA display epilogue (cf_resolve);
never used on the product path.  numpy float64 over an image of linear RGB,
returns RGBA8 as the 8-bit surface would store it (round to nearest).
"""
import numpy as np

INSET = np.array([[0.842479062253094, 0.0423282422610123, 0.0423756549057051],
                  [0.0784335999999992, 0.878468636469772, 0.0784336],
                  [0.0792237451477643, 0.0791661274605434, 0.879142973793104]]).T  # columns -> matrix
OUTSET = np.array([[1.1968790051, -0.0528968518, -0.0529716355],
                   [-0.0980208811, 1.1519031299, -0.0980434501],
                   [-0.0990297441, -0.0989611768, 1.1510736726]]).T
LUMA = np.array([0.2126, 0.7152, 0.0722])


def aces(c):  # resolve.wgsl:23-26
    a, b, cc, d, e = 2.51, 0.03, 2.43, 0.59, 0.14
    return np.clip((c * (a * c + b)) / (c * (cc * c + d) + e), 0.0, 1.0)


def agx(c):  # resolve.wgsl:28-50
    min_ev, max_ev = -12.47393, 4.026069
    v = np.maximum(c, 1e-10) @ INSET.T
    v = np.clip(np.log2(v), min_ev, max_ev)
    v = (v - min_ev) / (max_ev - min_ev)
    x2 = v * v
    x4 = x2 * x2
    v = 15.5 * x4 * x2 - 40.14 * x4 * v + 31.96 * x4 - 6.868 * x2 * v + 0.4298 * x2 + 0.1191 * v - 0.00232
    v = np.clip(v, 0.0, 1.0)
    luma = v @ LUMA
    v = v ** 1.35
    v = luma[..., None] + 1.4 * (v - luma[..., None])
    v = np.clip(v, 0.0, 1.0) @ OUTSET.T
    return np.clip(v, 0.0, 1.0) ** 2.2


def to_srgb(c):  # resolve.wgsl:52-56
    return np.where(c <= 0.0031308, c * 12.92, 1.055 * np.power(np.maximum(c, 0.0), 1.0 / 2.4) - 0.055)


def hash12(px, py):  # resolve.wgsl:58-62, in f32 with one rounding per operation
    f = np.float32
    px, py = np.asarray(px, f), np.asarray(py, f)
    fract = lambda x: (x - np.floor(x)).astype(f)  # noqa: E731
    qx, qy = fract(px * f(0.1031)), fract(py * f(0.1030))
    d = (qx * (qy + f(33.33))).astype(f) + (qy * (qx + f(33.33))).astype(f)
    qx, qy = (qx + d).astype(f), (qy + d).astype(f)
    return fract(((qx + qy).astype(f) * qx).astype(f)).astype(np.float64)


def smoothstep(e0, e1, x):
    t = np.clip((x - e0) / (e1 - e0), 0.0, 1.0)
    return t * t * (3.0 - 2.0 * t)


def resolve(rgb, scale=1.0, exposure_ev=0.0, bloom=0.0, grain=0.0, vignette=0.0, sharpen=0.0, agx_on=True):
    """rgb: (h, w, 3) linear RGB -> (h, w, 4) uint8 (resolve.wgsl:76-121)."""
    h, w, _ = rgb.shape
    img = np.asarray(rgb, np.float64) * scale
    exposure = 2.0 ** exposure_ev
    ys, xs = np.mgrid[0:h, 0:w]

    def load(dx, dy):
        return img[np.clip(ys + dy, 0, h - 1), np.clip(xs + dx, 0, w - 1)]

    c = img * exposure
    if bloom > 0:
        radius = max(h * 0.02, 4.0)
        glow, wsum = np.zeros_like(c), 0.0
        for k in range(32):
            fk = k + 0.5
            r = radius * np.sqrt(fk / 32.0)
            ang = fk * 2.399963
            ox, oy = int(np.cos(ang) * r), int(np.sin(ang) * r)
            s = load(ox, oy) * exposure
            lv = s @ LUMA
            wk = 1.0 - fk / 33.0
            glow += s * (np.maximum(lv - 1.6, 0.0) / np.maximum(lv, 1e-4) * wk)[..., None]
            wsum += wk
        c = c + bloom * 0.35 * glow / wsum
    if sharpen > 0:
        blur = (load(1, 0) + load(-1, 0) + load(0, 1) + load(0, -1)) * exposure * 0.25
        c = np.maximum(c + sharpen * (load(0, 0) * exposure - blur), 0.0)
    px, py = xs + 0.5, ys + 0.5
    ux, uy = px / w - 0.5, py / h - 0.5
    c = c * (1.0 - vignette * smoothstep(0.15, 0.75, (ux * ux + uy * uy) * 2.0))[..., None]
    m = agx(c) if agx_on else aces(c)
    if grain > 0:
        g = (hash12(np.float32(px) + np.float32(0.37), np.float32(py) + np.float32(0.11)) - 0.5) * 2.0
        shade = 1.0 - smoothstep(0.0, 1.0, m @ LUMA)
        m = np.clip(m + (g * grain * (0.35 + 0.65 * shade))[..., None], 0.0, 1.0)
    out = np.empty((h, w, 4), np.uint8)
    out[..., :3] = np.rint(np.clip(to_srgb(m), 0.0, 1.0) * 255.0).astype(np.uint8)
    out[..., 3] = 255
    return out
