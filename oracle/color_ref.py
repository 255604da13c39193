"""The reference's colour-matching helpers in numpy f32, for the table tests.

TEST INFRASTRUCTURE: used only by tests/ as the checker of the committed
colour tables (canvaz_film/data/reference_tables.npz).  Each function follows
the named reference function statement by statement, one f32 rounding per
operation:
  - reflectance_of   src/color/mod.rs:46-100 (sRGB -> 16-band reflectance:
                     a red / green / blue logistic basis over the band centres,
                     fitted to the target XYZ by Cramer's rule, 6 corrections)
  - band_wavelengths src/color/mod.rs:102-108
  - xyz_to_srgb      src/color/mod.rs:320-333 (the matrix km.wgsl:51-62 uses,
                     then the sRGB encode)
"""
import numpy as np

f32 = np.float32
NBAND = 16


def _dec(c):
    c = f32(c)
    return f32(c / f32(12.92)) if c <= f32(0.04045) else f32(np.power(f32((c + f32(0.055)) / f32(1.055)), f32(2.4)))


def band_wavelengths():
    return [f32(f32(410.0) + f32(20.0) * f32(b)) for b in range(NBAND)]


def _det(a):
    return f32(f32(f32(a[0][0] * f32(f32(a[1][1] * a[2][2]) - f32(a[1][2] * a[2][1])))
                   - f32(a[0][1] * f32(f32(a[1][0] * a[2][2]) - f32(a[1][2] * a[2][0]))))
               + f32(a[0][2] * f32(f32(a[1][0] * a[2][1]) - f32(a[1][1] * a[2][0]))))


def _solve(m, v):
    d = _det(m)
    out = [f32(0)] * 3
    for c in range(3):
        a = [list(r) for r in m]
        for i in range(3):
            a[i][c] = v[i]
        out[c] = f32(_det(a) / d) if abs(d) > 1e-12 else f32(0)
    return out


def reflectance_of(srgb, cmf):
    """src/color/mod.rs:46-100."""
    cmf = np.asarray(cmf, f32)
    lin = [_dec(c) for c in srgb]
    M = [[f32(0.4124), f32(0.3576), f32(0.1805)], [f32(0.2126), f32(0.7152), f32(0.0722)],
         [f32(0.0193), f32(0.1192), f32(0.9505)]]
    target = [f32(f32(f32(M[i][0] * lin[0]) + f32(M[i][1] * lin[1])) + f32(M[i][2] * lin[2])) for i in range(3)]
    basis = []
    for lam in band_wavelengths():
        blue = f32(f32(1) / f32(f32(1) + f32(np.exp(f32(f32(lam - f32(490)) / f32(18))))))
        red = f32(f32(1) / f32(f32(1) + f32(np.exp(f32(-f32(lam - f32(585)) / f32(18))))))
        basis.append([red, max(f32(f32(f32(1) - blue) - red), f32(0)), blue])
    m = [[f32(0)] * 3 for _ in range(3)]
    for b in range(NBAND):
        for i in range(3):
            for c in range(3):
                m[i][c] = f32(m[i][c] + f32(basis[b][c] * cmf[b * 3 + i]))
    want = list(target)
    refl = [f32(0)] * NBAND
    for _ in range(6):
        k = _solve(m, want)
        for b in range(NBAND):
            v = f32(f32(f32(basis[b][0] * k[0]) + f32(basis[b][1] * k[1])) + f32(basis[b][2] * k[2]))
            refl[b] = f32(min(max(v, f32(0.005)), f32(0.97)))
        got = [f32(0)] * 3
        for b in range(NBAND):
            for i in range(3):
                got[i] = f32(got[i] + f32(refl[b] * cmf[b * 3 + i]))
        for i in range(3):
            want[i] = f32(want[i] + f32(target[i] - got[i]))
    return np.array(refl, f32)


def xyz_to_srgb(xyz):
    """src/color/mod.rs:320-333."""
    x, y, z = (f32(v) for v in xyz)
    r = f32(f32(f32(f32(3.2406) * x) - f32(f32(1.5372) * y)) - f32(f32(0.4986) * z))
    g = f32(f32(f32(f32(-0.9689) * x) + f32(f32(1.8758) * y)) + f32(f32(0.0415) * z))
    b = f32(f32(f32(f32(0.0557) * x) - f32(f32(0.2040) * y)) + f32(f32(1.0570) * z))

    def enc(c):
        c = min(max(c, f32(0)), f32(1))
        if c <= f32(0.0031308):
            return f32(f32(12.92) * c)
        return f32(f32(f32(1.055) * f32(np.power(c, f32(f32(1.0) / f32(2.4))))) - f32(0.055))
    return np.array([enc(r), enc(g), enc(b)], f32)
