"""CPU restatement of the render pass's reading of the film (TEST
INFRASTRUCTURE: only tests/ use it, as the checker).

numpy over many canvas points, in float64, following shaders/render.wgsl
with the plain camera (no beauty mode, colour plane at the film's
resolution):
  surf_at :305-312, surf_cubic :335-353, cr_w :328-333,
  wet_at :355-361, wet_bilinear :394-406, col_at :644-652,
  color_sharp :706-750, base_slope :628-638; the key-light shadow march
  surf_bilinear :314-326, shadow_at :846-866 (surf_march = surf_bilinear).
Pinned by tests/golden/relief_samples.npz, which the reference's own shader
functions (mechanically translated, oracle/wgsl_ref) wrote.
"""
import numpy as np


def f(v):
    """A literal of the shader: f32 (the translated reference widens them so)."""
    return float(np.float32(v))


class Relief:
    def __init__(self, w, h, width_m, height_m, hplane, mplane, rgba):
        self.w, self.h = w, h
        self.wm, self.hm = f(width_m), f(height_m)
        self.dx = float(np.float32(width_m) / np.float32(w))
        self.hp = np.asarray(hplane, np.float64).reshape(h, w)
        self.mp = np.asarray(mplane, np.float64).reshape(h, w)
        self.col = np.asarray(rgba, np.float64).reshape(h, w, 4)

    def _clamp(self, i, j):
        return np.clip(j, 0, self.h - 1), np.clip(i, 0, self.w - 1)

    def surf_at(self, i, j):
        jj, ii = self._clamp(i, j)
        return self.hp[jj, ii] + self.mp[jj, ii]

    def wet_at(self, i, j):
        jj, ii = self._clamp(i, j)
        return self.hp[jj, ii]

    def col_at(self, i, j):
        jj, ii = self._clamp(i, j)
        return self.col[jj, ii]

    @staticmethod
    def cr_w(t):
        t2 = t * t
        t3 = t2 * t
        u = 1.0 - t
        return np.stack([u * u * u, 3.0 * t3 - 6.0 * t2 + 4.0, -3.0 * t3 + 3.0 * t2 + 3.0 * t + 1.0, t3]) / 6.0

    def _grid(self, px, py):
        gx, gy = px / self.dx - 0.5, py / self.dx - 0.5
        fx, fy = np.floor(gx), np.floor(gy)
        return fx.astype(np.int64), fy.astype(np.int64), gx - fx, gy - fy

    def outside(self, px, py):
        return (px < 0) | (py < 0) | (px > self.wm) | (py > self.hm)

    def surf_cubic(self, px, py):
        i, j, tx, ty = self._grid(px, py)
        wx, wy = self.cr_w(tx), self.cr_w(ty)
        s = np.zeros_like(px)
        for b in range(-1, 3):
            row = np.zeros_like(px)
            for a in range(-1, 3):
                row = row + wx[a + 1] * self.surf_at(i + a, j + b)
            s = s + wy[b + 1] * row
        return np.where(self.outside(px, py), 0.0, np.maximum(s, 0.0))

    def wet_bilinear(self, px, py):
        i, j, tx, ty = self._grid(px, py)
        a, b, c, d = self.wet_at(i, j), self.wet_at(i + 1, j), self.wet_at(i, j + 1), self.wet_at(i + 1, j + 1)
        r0, r1 = a * (1 - tx) + b * tx, c * (1 - tx) + d * tx
        return np.where(self.outside(px, py), 0.0, r0 * (1 - ty) + r1 * ty)

    def surf_bilinear(self, px, py):
        i, j, tx, ty = self._grid(px, py)
        a, b, c, d = self.surf_at(i, j), self.surf_at(i + 1, j), self.surf_at(i, j + 1), self.surf_at(i + 1, j + 1)
        r0, r1 = a * (1 - tx) + b * tx, c * (1 - tx) + d * tx
        return np.where(self.outside(px, py), 0.0, r0 * (1 - ty) + r1 * ty)

    def shadow_at(self, px, py, z0, light, top):
        """shadow_at with the plain camera: 20 steps of 1.5 cells toward the
        light over the bilinear relief, stopping where the ray rises above
        `top` (cam.canvas.w); 1 - the deepest penetration over its penumbra."""
        lx, ly, lz = (float(v) for v in light)
        if lz <= f(0.05):
            return np.ones_like(px)
        step = self.dx * 1.5
        spread = np.tan(f(0.12))  # tan(KEY_HALF_ANGLE)
        sh = np.ones_like(px)
        live = np.ones(px.shape, bool)
        for k in range(1, 21):
            d = float(k) * step
            zs = self.surf_bilinear(px + lx / lz * d, py + ly / lz * d)
            zr = z0 + d
            live &= ~(zr > float(top))
            pen = d * spread / lz + 0.5 * step
            sh = np.where(live, np.minimum(sh, 1.0 - np.clip((zs - zr) / pen, 0.0, 1.0)), sh)
        return sh

    def shadow(self, pts, z0, light, top):
        """The 2 values per point of cf_relief_shadow: surf_bilinear, shadow_at."""
        pts = np.asarray(pts, np.float64).reshape(-1, 2)
        px, py = pts[:, 0], pts[:, 1]
        return np.column_stack([self.surf_bilinear(px, py),
                                self.shadow_at(px, py, np.asarray(z0, np.float64), light, top)])

    def base_slope(self, px, py):
        e = f(0.7) * self.dx
        sx = self.surf_cubic(px + e, py) - self.surf_cubic(px - e, py)
        sy = self.surf_cubic(px, py + e) - self.surf_cubic(px, py - e)
        return sx / (2.0 * e), sy / (2.0 * e)

    @staticmethod
    def smoothstep(e0, e1, x):
        t = np.clip((x - e0) / (e1 - e0), 0.0, 1.0)
        return t * t * (3.0 - 2.0 * t)

    def color_sharp(self, px, py):
        i, j, tx, ty = self._grid(px, py)
        wb = [(1 - tx) * (1 - ty), tx * (1 - ty), (1 - tx) * ty, tx * ty]
        hw = [self.wet_at(i, j), self.wet_at(i + 1, j), self.wet_at(i, j + 1), self.wet_at(i + 1, j + 1)]
        cs = [self.col_at(i, j), self.col_at(i + 1, j), self.col_at(i, j + 1), self.col_at(i + 1, j + 1)]
        cbil = wb[0][:, None] * cs[0] + wb[1][:, None] * cs[1] + wb[2][:, None] * cs[2] + wb[3][:, None] * cs[3]
        hmax = np.maximum(np.maximum(hw[0], hw[1]), np.maximum(hw[2], hw[3]))
        hmin = np.minimum(np.minimum(hw[0], hw[1]), np.minimum(hw[2], hw[3]))
        with np.errstate(divide="ignore", invalid="ignore"):
            edge = self.smoothstep(f(0.3), f(0.6), 1.0 - hmin / hmax)
        wx, wy = self.cr_w(tx), self.cr_w(ty)
        hb = np.zeros_like(px)
        hb2 = np.zeros_like(px)
        for b in range(-1, 3):
            for a in range(-1, 3):
                wv = wx[a + 1] * wy[b + 1]
                hv = self.wet_at(i + a, j + b)
                hb = hb + wv * hv
                hb2 = hb2 + wv * hv * hv
        hb = np.maximum(hb, 0.0)
        hin = hb2 / np.maximum(hb, f(1e-9))
        win = [wb[k] * hw[k] for k in range(4)]
        wout = [wb[k] * (hmax - hw[k]) for k in range(4)]
        sin = np.maximum(win[0] + win[1] + win[2] + win[3], f(1e-12))
        sout = np.maximum(wout[0] + wout[1] + wout[2] + wout[3], f(1e-12))
        cin = (win[0][:, None] * cs[0] + win[1][:, None] * cs[1] + win[2][:, None] * cs[2] + win[3][:, None] * cs[3])
        cout = (wout[0][:, None] * cs[0] + wout[1][:, None] * cs[1] + wout[2][:, None] * cs[2]
                + wout[3][:, None] * cs[3])
        cin = cin / sin[:, None]
        cout = cout / sout[:, None]
        s = self.smoothstep(0.25, f(0.45), hb / np.maximum(hin, f(1e-9)))
        ce = cout * (1 - s)[:, None] + cin * s[:, None]
        mixed = cbil * (1 - edge)[:, None] + ce * edge[:, None]
        mixed[:, 3] = cbil[:, 3]
        plain = (hmax <= f(1e-6)) | ~(edge > 0)
        return np.where(plain[:, None], cbil, mixed)

    def sample(self, pts):
        """The 8 values per point of cf_sample_relief."""
        pts = np.asarray(pts, np.float64).reshape(-1, 2)
        px, py = pts[:, 0], pts[:, 1]
        sx, sy = self.base_slope(px, py)
        col = self.color_sharp(px, py)
        return np.column_stack([self.surf_cubic(px, py), sx, sy, col, self.wet_bilinear(px, py)])
