"""Generates the golden fixtures tests/golden/*.npz.

Runs where the reference checkout exists (REFERENCE, else where
oracle/wgsl_ref/build_ref.py's reference_root finds it):
  1. oracle/wgsl_ref/build_ref.py translates the reference WGSL to C++ and
     builds oracle/_ref/libwgslref.so;
  2. each case below is a small seeded canvas; its frame schedule (frame dt,
     substeps) and packed Params come from the oracle's update_params /
     choose_substeps restatement;
  3. the translated reference steps the frames (FP64), and the inputs, the
     schedule and the reference's final planes are stored.
tests/test_golden.py replays every fixture through the oracle.

Usage: python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "paint-sim-3d_gb300"))

OUT_FIELDS = ["h", "m", "rheo", "strata_h", "strata_pig", "strata_cure", "sub_refl", "delta", "fnorm",
              "color", "acc", "tile_flags", "pres", "flux", "alpha", "tmp", "acc_s", "alpha_s", "lay"]


def mixed_canvas(seed):
    """Blob canvas with multi-strata stacks, thinner, pigment-table viscosity
    (slot 14 = 0) in some strata, weave relief and partial cure."""
    from canvaz_film import synth
    cv = synth.blob_canvas(48, 48, seed, n_blobs=8, sigma=(3, 9), per_cell_n=False, tables="reference")
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    p = cv.planes
    n = cv.n
    wet = p["h"] > 0
    k = rng.integers(1, 5, n)
    frac = rng.dirichlet(np.ones(4), n).astype(np.float32)
    for s in range(4):
        use = wet & (k > s)
        p["strata_h"][:, s] = np.where(use, 0.0, p["strata_h"][:, s])
    tot = np.zeros(n, np.float32)
    for s in range(4):
        tot += np.where(wet & (k > s), frac[:, s], 0)
    for s in range(4):
        use = wet & (k > s)
        p["strata_h"][:, s] = np.where(use, p["h"] * frac[:, s] / np.maximum(tot, 1e-9), 0)
        pig = rng.dirichlet(np.full(12, 0.5), n).astype(np.float32)
        p["strata_pig"][:, 16 * s:16 * s + 12] = np.where(use[:, None], pig, 0)
        p["strata_pig"][:, 16 * s + 12] = np.where(use, rng.uniform(0, 0.3, n) * (rng.random(n) < 0.3), 0)
        p["strata_pig"][:, 16 * s + 13] = np.where(use, rng.uniform(0, 2, n), 0)
        lm = rng.uniform(np.log(0.05), np.log(2.0), n) + 10
        p["strata_pig"][:, 16 * s + 14] = np.where(use & (rng.random(n) < 0.7), lm, 0)
        p["strata_cure"][:, s] = np.where(use, rng.uniform(0, 0.5, n), 0)
    p["lay"][:] = rng.integers(0, 2 ** 24, n, dtype=np.uint32)
    cv.settings.update(weave_um=25.0, kline=0.5, debug_view=0, hyst_deg=10.0)
    return cv


def cases():
    from canvaz_film import synth
    out = []
    cv = synth.blob_canvas(48, 48, 11, n_blobs=6, sigma=(3, 10), per_cell_n=False, tables="reference",
                           tau=(0.0, 1.0), mu=(0.05, 0.5))
    cv.settings.update(rho=1000.0, sigma=0.035)
    out.append(("blob_frame60", cv, dict(frame_dt=1 / 60, frames=5, adaptive_substeps=True)))
    cv = synth.drip_canvas(64, 64, 5, n_lines=6, per_cell_n=False)
    out.append(("drip_tilt", cv, dict(frame_dt=2e-4, frames=12, substeps=1)))
    cv = mixed_canvas(21)
    out.append(("mixed_stack", cv, dict(frame_dt=1 / 60, frames=6, adaptive_substeps=True)))
    cv = mixed_canvas(31)
    cv.settings.update(cure_rate=40.0, weave_um=0.0, kline=0.0)
    out.append(("cure_commit", cv, dict(frame_dt=1 / 60, frames=4, substeps=2)))
    cv = synth.drip_canvas(48, 48, 7, n_lines=5, per_cell_n=False, tilt_deg=35.0)
    cv.settings.update(no_transl=1, no_shape=1, no_hold=1, debug_view=1, tilt_dir_deg=20.0)
    out.append(("toggles_debug", cv, dict(frame_dt=5e-4, frames=8, substeps=1)))
    cv = synth.blob_canvas(40, 40, 9, n_blobs=5, sigma=(3, 8), per_cell_n=False, tau=(0, 3), mu=(0.1, 2))
    cv.settings.update(all_active=0, n_index=0.7, contact_angle_deg=60.0)
    out.append(("shear_thinning", cv, dict(frame_dt=1 / 60, frames=5, adaptive_substeps=True)))
    cv = synth.blob_canvas(48, 40, 13, n_blobs=5, sigma=(3, 8), per_cell_n=False, tau=(0, 0.5), mu=(0.05, 0.3),
                           peak_mm=(1.0, 3.0))
    out.append(("spreading_front", cv, dict(frame_dt=1 / 60, frames=10, adaptive_substeps=True)))
    cv = synth.blob_canvas(48, 48, 17, n_blobs=4, sigma=(3, 8), per_cell_n=False, tables="reference",
                           tau=(0.0, 1.0), mu=(0.05, 0.5))
    out.append(("deposit_strokes", cv, dict(frame_dt=1 / 60, frames=5, adaptive_substeps=True,
                                            deposits={0: deposit_set(cv, 5), 2: deposit_set(cv, 6)})))
    cv = synth.blob_canvas(48, 48, 17, n_blobs=1, sigma=(2, 5), per_cell_n=False, tables="reference",
                           tau=(0.0, 1.0), mu=(0.05, 0.5))
    out.append(("deposit_fresh", cv, dict(frame_dt=1 / 60, frames=4, adaptive_substeps=True,
                                          deposits={0: deposit_set(cv, 100), 2: deposit_set(cv, 102)})))
    cv = synth.blob_canvas(48, 48, 29, n_blobs=4, sigma=(4, 9), per_cell_n=False, tables="reference",
                           tau=(0.0, 0.3), mu=(0.05, 0.2), peak_mm=(3.0, 5.0))
    cv.settings.update(implicit_hydro=1)
    out.append(("implicit_pour", cv, dict(frame_dt=1 / 60, frames=4, adaptive_substeps=True)))
    return out


def deposit_set(cv, seed):
    """Strokes, capsules, a dot, an angled ribbon, a recycled deposit and one
    that crosses the canvas edge, built by the Deposit constructors."""
    import deposit_ref as dr
    w = np.float32(cv.settings["width_m"])
    dx = w / np.float32(cv.w)
    rng = np.random.Generator(np.random.PCG64(seed))

    def pig():
        v = np.zeros(16)
        v[:12] = rng.dirichlet(np.full(12, 0.5))
        v[13] = rng.uniform(0.5, 2.0)
        v[14] = rng.uniform(9.0, 11.0) if rng.random() < 0.5 else 0.0
        return dr.pack_pig(v)

    def pt():
        return (float(rng.uniform(0.1, 0.9) * w), float(rng.uniform(0.1, 0.9) * w))

    deps = []
    for _ in range(3):
        a = pt()
        b = (a[0] + float(rng.uniform(-0.3, 0.3) * w), a[1] + float(rng.uniform(-0.3, 0.3) * w))
        deps.append(dr.stroke(a, b, float(rng.uniform(1.5, 4) * dx), float(rng.uniform(0.5, 3) * 1e-9), pig(), dx))
    a = pt()
    deps.append(dr.capsule(a, (a[0] + float(2 * dx), a[1] - float(3 * dx)), float(2.5 * dx), 1e-9, pig(), dx))
    deps.append(dr.capsule(pt(), pt(), float(1.2 * dx), 0.7e-9, pig(), dx))
    a = pt()
    deps.append(dr.capsule(a, a, float(3 * dx), 1.5e-9, pig(), dx))
    a = pt()
    deps.append(dr.ribbon(a, (a[0] + float(6 * dx), a[1] + float(2 * dx)), (np.cos(0.3), -np.sin(0.3)),
                          (np.cos(0.4), np.sin(0.4)), float(2 * dx), float(3.5 * dx), 0, 1.2e-9, pig(), dx))
    d = dr.stroke((float(-2 * dx), float(0.5 * w)), (float(5 * dx), float(0.55 * w)), float(2 * dx), 1e-9, pig(), dx)
    d["kind"] |= dr.RECYCLED
    deps.append(d)
    for k, d in enumerate(deps):
        d["kind"] |= ((k % 6) + 1) << dr.METHOD_SHIFT
    return np.array(deps)


def main():
    sys.path.insert(0, str(ROOT / "oracle" / "wgsl_ref"))
    import build_ref
    ref = str(build_ref.reference_root())
    subprocess.run([sys.executable, str(ROOT / "oracle" / "wgsl_ref" / "build_ref.py"), ref], check=True)
    import pyoracle as po
    po.build()
    for name, cv, sched in cases():
        st = po.make_settings(cv.settings)
        o = po.Oracle(cv.w, cv.h, st, 0, 64)
        o.set_tables(cv.pigtab, cv.cmf)
        o.write_state(cv.planes)
        r = po.RefShaders(cv.w, cv.h)
        r.set_tables(cv.pigtab, cv.cmf)
        r.write_state(cv.planes)
        schedule, params, dep_frames, implicit = [], [], {}, []
        for f in range(sched["frames"]):
            fdt = sched["frame_dt"]
            if f in sched.get("deposits", {}):
                import deposit_ref as dr
                deps = sched["deposits"][f]
                hm, hp = o.host_stats()
                _, start, cnt, items, _, _ = dr.bin_deposits(deps, cv.w, cv.h, st.width_m, st.height_m, hm, hp)
                o.upload_deposits(deps)
                r.set_deposits(deps, start, cnt, items)
                dep_frames["deposits_%d" % f] = deps.view(np.uint8).reshape(len(deps), 96)
            n = o.choose_substeps(fdt) if sched.get("adaptive_substeps") else sched["substeps"]
            o.update_params(fdt, n)
            p = o.params()
            r.set_params(p)
            r.set_implicit(o.implicit_steps(), st.implicit_iters)
            implicit.append(o.implicit_steps())
            r.encode_frame(n)
            o.encode_frame(n)
            schedule.append((fdt, n))
            params.append(np.frombuffer(bytes(p), np.uint8))
        outs = {"out_" + k: r.buf(k) for k in OUT_FIELDS}
        worst = max(float(np.abs(o.buf(k) - outs["out_" + k]).max()) for k in OUT_FIELDS if k not in ("rheo", "lay"))
        assert np.array_equal(o.buf("lay"), outs["out_lay"]), "lay differs"
        ins = {"in_" + k: np.asarray(v) for k, v in cv.planes.items()}
        np.savez_compressed(HERE / ("%s.npz" % name), w=cv.w, h=cv.h, settings=json.dumps(cv.settings),
                            pigtab=cv.pigtab, cmf=cv.cmf, schedule=np.array(schedule),
                            params=np.stack(params), implicit_steps=np.array(implicit), **ins, **outs,
                            **dep_frames)
        print("%-16s %dx%d frames %d substeps %s implicit %s  oracle-vs-ref max |d| %.3e" % (
            name, cv.w, cv.h, len(schedule), [s[1] for s in schedule], implicit, worst))


if __name__ == "__main__":
    main()
