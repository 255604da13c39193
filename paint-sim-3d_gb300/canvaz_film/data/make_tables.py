"""Derives the reference's colour tables into reference_tables.npz.

Reads, from a checkout of the reference (default: the REFERENCE env var),
  - the CIE 1931 CMF and D65 arrays of src/color/mod.rs:110-148 and folds them
    into 16 bands exactly as cmf_table (src/color/mod.rs:150-171) does, in f32;
  - the 12 pigments of assets/pigments.ron (what load_pigments,
    src/color/mod.rs:226-241, returns when the file parses) and packs them as
    pigment_table (src/color/mod.rs:243-258): K = (1-r)^2/(2r) * scatter,
    S = scatter per band, viscosity at 32, yield at 33, tint at 34.
The npz is committed; this script is only rerun where the reference exists.
Usage: python make_tables.py [reference_root]
"""
import os
import re
import sys
from pathlib import Path

import numpy as np

f32 = np.float32


def parse_rust_f32_array(txt, name):
    m = re.search(r"const %s:[^=]*=\s*\[(.*?)\];" % name, txt, re.S)
    body = m.group(1)
    rows = re.findall(r"\[([^\[\]]*)\]", body)
    if rows:
        return [[float(x) for x in r.split(",") if x.strip()] for r in rows]
    return [float(x) for x in body.replace("\n", " ").split(",") if x.strip()]


def cmf_table(ref):
    txt = (ref / "src/color/mod.rs").read_text()
    cmf = parse_rust_f32_array(txt, "CMF")
    d65 = parse_rust_f32_array(txt, "D65")
    t = np.zeros(48, dtype=f32)
    ysum = f32(0)
    for b in range(16):
        acc = [f32(0)] * 3
        for s in range(2):
            k = 2 * b + s
            w = f32(d65[k])
            for c in range(3):
                acc[c] = f32(acc[c] + f32(f32(cmf[k][c + 1]) * w))
        for c in range(3):
            t[b * 3 + c] = acc[c]
        ysum = f32(ysum + acc[1])
    return (t / ysum).astype(f32)


def pigment_table(ref):
    txt = (ref / "assets/pigments.ron").read_text()
    blocks = re.findall(r"\(\s*name:\s*\"([^\"]+)\"(.*?)\)\s*,?\s*(?=\(\s*name:|\]\s*,?\s*\))", txt, re.S)
    assert len(blocks) == 12, len(blocks)
    t = np.zeros(12 * 40, dtype=f32)
    names = []
    for i, (name, body) in enumerate(blocks):
        names.append(name)
        refl = [f32(x) for x in re.search(r"reflectance:\s*\[(.*?)\]", body, re.S).group(1).replace("\n", " ").split(",") if x.strip()]
        scatter = f32(float(re.search(r"scatter:\s*([0-9.eE+-]+)", body).group(1)))
        tm = re.search(r"tint:\s*([0-9.eE+-]+)", body)
        tint = f32(float(tm.group(1))) if tm else f32(1.0)
        visc = f32(float(re.search(r"viscosity:\s*([0-9.eE+-]+)", body).group(1)))
        yld = f32(float(re.search(r"yield_stress:\s*([0-9.eE+-]+)", body).group(1)))
        for b in range(16):
            r = min(max(refl[b], f32(0.01)), f32(0.98))
            ks = f32(f32(f32(1) - r) * f32(f32(1) - r)) / f32(f32(2) * r)
            t[i * 40 + b] = f32(ks * scatter)
            t[i * 40 + 16 + b] = scatter
        t[i * 40 + 32] = visc
        t[i * 40 + 33] = yld
        t[i * 40 + 34] = tint
    return t, names


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE")
    if not root:
        sys.exit("usage: make_tables.py REFERENCE_ROOT (or set REFERENCE)")
    ref = Path(root)
    cmf = cmf_table(ref)
    pig, names = pigment_table(ref)
    out = Path(__file__).with_name("reference_tables.npz")
    np.savez(out, cmf=cmf, pigtab=pig, names=np.array(names))
    print("wrote", out, cmf[:6], pig[:3])


if __name__ == "__main__":
    main()
