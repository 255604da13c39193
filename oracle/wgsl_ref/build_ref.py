"""Builds oracle/_ref/libwgslref.so from the reference shaders.

TEST INFRASTRUCTURE.  Needs the reference checkout (argument, else the
REFERENCE env var, else the checkout's mount point in the build container:
reference_root() below is the one place that names it); does nothing when it
is absent.  Steps:
translate.py writes oracle/_ref/ref_shaders.inc (FP64), then g++ compiles
driver.cpp against it; the relief and colour sampling of render.wgsl goes the
same way into render_ref.inc and librenderref.so (render_driver.cpp), and the
display fragment of resolve.wgsl into resolve_ref.inc and libresolveref.so
(resolve_driver.cpp).  Everything it writes stays in oracle/_ref/, which is
git-ignored.
Usage: python build_ref.py [reference_root]
"""
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"


# where the build container mounts the reference checkout (read-only)
_MOUNT = "/root/reference"


def reference_root(ref=None):
    """The reference checkout: `ref`, else $REFERENCE, else the mount point."""
    return Path(ref or os.environ.get("REFERENCE") or _MOUNT)


def build(ref=None):
    ref = reference_root(ref)
    if not (ref / "shaders" / "film.wgsl").exists():
        print("reference shaders not found at %s; skipping" % ref)
        return None
    OUT.mkdir(exist_ok=True)
    subprocess.run([sys.executable, str(HERE / "translate.py"), str(ref), str(OUT / "ref_shaders.inc"), "double"],
                   check=True)
    shutil.copy(HERE / "wgsl_rt_types.inc", OUT / "wgsl_rt_types.inc")
    lib = OUT / "libwgslref.so"
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(OUT), str(HERE / "driver.cpp"),
                    "-o", str(lib)], check=True)
    # the relief / colour sampling of render.wgsl (a subset: the beauty-mode
    # helpers it never reaches with the plain camera are stubs)
    sys.path.insert(0, str(HERE))
    import translate
    src = translate.translate_subset(str(ref), "render.wgsl",
                                     ["surf_cubic", "base_slope", "color_sharp", "wet_bilinear", "surf_bilinear",
                                      "shadow_at"],
                                     {"color_beauty", "color_crisp", "surf_smooth", "hwarp"}, "wgrr")
    (OUT / "render_ref.inc").write_text(src)
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(OUT), str(HERE / "render_driver.cpp"),
                    "-o", str(OUT / "librenderref.so")], check=True)
    # the renderer's whole fragment shader (fs, lit and all they reach), in
    # f32 as the shader computes (one rounding per operation: no contraction)
    src = translate.translate_subset(str(ref), "render.wgsl", ["fs"], set(), "wgrf", "float")
    (OUT / "render_fs_ref.inc").write_text(src)
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(OUT),
                    str(HERE / "render_fs_driver.cpp"), "-o", str(OUT / "librenderfsref.so")], check=True)
    # the display fragment of resolve.wgsl, in f32 as the shader computes
    # (one rounding per operation: no contraction), its uniform's fields a, b,
    # c kept as they are named
    src = translate.translate_subset(str(ref), "resolve.wgsl", ["fs"], set(), "wgres", "float", members={"R"})
    (OUT / "resolve_ref.inc").write_text(src)
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(OUT),
                    str(HERE / "resolve_driver.cpp"), "-o", str(OUT / "libresolveref.so")], check=True)
    return lib


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
