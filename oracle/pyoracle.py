"""ctypes wrappers of the oracle (liboracle.so) and of the translated
reference shaders (_ref/libwgslref.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  Never on the product path.
"""
import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT / "paint-sim-3d_gb300"))
from canvaz_film.capi import Params, Settings  # noqa: E402

LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libwgslref.so"

# name -> values per cell in the oracle layout
PLANES = {
    "h": 1, "m": 1, "rheo": 3, "strata_h": 4, "strata_cure": 4, "strata_pig": 64, "sub_refl": 16,
    "lay": 1, "pres": 2, "flux": 4, "acc": 4, "alpha": 1, "tmp": 1, "acc_s": 16, "alpha_s": 4,
    "strata_h2": 4, "strata_cure2": 4, "strata_pig2": 64, "h_frame": 1, "fnorm": 2, "delta": 1,
    "color": 4, "detail": 4,
}
STATE = ["h", "m", "rheo", "strata_h", "strata_pig", "strata_cure", "sub_refl", "lay"]
KERNELS = ["mark_tiles", "compact_tiles", "cure_step", "clear_acc", "laplacian", "plug", "fluxes",
           "limiter", "apply", "nose", "strata_split", "reduce_tiles", "strata_limit", "strata_update",
           "strata_copy_back", "strata_fill", "shade_full"]


def build(force=False):
    """Compiles the oracle (g++ -O2 -fopenmp -ffp-contract=off) into
    oracle/_build/liboracle.so."""
    src = [HERE / "oracle_capi.cpp", HERE / "film_oracle.hpp", ROOT / "include" / "canvaz_film.h"]
    if LIB.exists() and not force and all(LIB.stat().st_mtime >= s.stat().st_mtime for s in src):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    # one rounding per operation on every host (gcc contracts a * b + c into
    # a fused multiply-add by default where the ISA has one, as on aarch64)
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           str(HERE / "oracle_capi.cpp"), "-o", str(LIB) + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp = C.c_void_p
        L.cfo_create.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(Settings), C.c_int, C.c_int]
        L.cfo_create.restype = vp
        L.cfo_destroy.argtypes = [vp]
        L.cfo_set_tables.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.cfo_update_params.argtypes = [vp, C.c_float, C.c_uint32]
        L.cfo_get_params.argtypes = [vp, C.POINTER(Params), C.POINTER(C.c_uint32)]
        L.cfo_set_params.argtypes = [vp, C.POINTER(Params)]
        L.cfo_choose_substeps.argtypes = [vp, C.c_float]
        L.cfo_choose_substeps.restype = C.c_uint32
        L.cfo_after_write_state.argtypes = [vp]
        L.cfo_encode_frame.argtypes = [vp, C.c_uint32]
        L.cfo_step_adaptive.argtypes = [vp, C.c_float]
        L.cfo_step_adaptive.restype = C.c_float
        L.cfo_dry_now.argtypes = [vp]
        L.cfo_stats.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_uint32),
                                C.POINTER(C.c_double)]
        u32p = C.POINTER(C.c_uint32)
        L.cfo_set_deposits.argtypes = [vp, C.c_void_p, C.c_uint32, u32p, u32p, C.c_uint32, u32p, C.c_uint32,
                                       C.c_float]
        L.cfo_host_stats.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.cfo_run.argtypes = [vp, C.c_char_p]
        L.cfo_run.restype = C.c_int
        L.cfo_buffer_len.argtypes = [vp, C.c_char_p]
        L.cfo_buffer_len.restype = C.c_size_t
        L.cfo_buffer.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double), C.c_int]
        L.cfo_buffer.restype = C.c_int
        _lib = L
    return _lib


def _f32p(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


class Oracle:
    """The oracle film: FP64 (bits=64) or the FP32 mirror (bits=32)."""

    def __init__(self, w, h, settings, pig_mode=0, bits=64):
        self.w, self.h, self.n = w, h, w * h
        self.L = lib()
        self.settings = settings
        self.p = self.L.cfo_create(w, h, C.byref(settings), pig_mode, bits)

    def __del__(self):
        if getattr(self, "p", None):
            self.L.cfo_destroy(self.p)
            self.p = None

    def set_tables(self, pigtab, cmf):
        a, pa = _f32p(pigtab)
        b, pb = _f32p(cmf)
        self.L.cfo_set_tables(self.p, pa, pb)

    def buf(self, name):
        n = self.L.cfo_buffer_len(self.p, name.encode())
        out = np.zeros(n, np.float64)
        assert self.L.cfo_buffer(self.p, name.encode(), out.ctypes.data_as(C.POINTER(C.c_double)), 0)
        return out

    def set_buf(self, name, values):
        n = self.L.cfo_buffer_len(self.p, name.encode())
        v = np.ascontiguousarray(np.asarray(values, np.float64).reshape(-1))
        assert v.size == n, (name, v.size, n)
        assert self.L.cfo_buffer(self.p, name.encode(), v.ctypes.data_as(C.POINTER(C.c_double)), 1)

    def write_state(self, planes):
        """Film::write_state: the eight planes, then scratch clearing and stats."""
        for k in STATE:
            v = np.asarray(planes[k])
            if k == "rheo":
                r = np.zeros((self.n, 3))
                r[:, :2] = v.reshape(self.n, 2)
                r[:, 2] = self.settings.n_index
                v = r
            self.set_buf(k, v)
        self.L.cfo_after_write_state(self.p)

    def update_params(self, frame_dt, substeps):
        self.L.cfo_update_params(self.p, frame_dt, substeps)

    def params(self):
        p = Params()
        n = C.c_uint32()
        self.L.cfo_get_params(self.p, C.byref(p), C.byref(n))
        return p

    def set_params(self, p):
        self.L.cfo_set_params(self.p, C.byref(p))

    def implicit_steps(self):
        """Film::implicit_steps of the last update_params (0 with implicit_hydro off)."""
        p, n = Params(), C.c_uint32()
        self.L.cfo_get_params(self.p, C.byref(p), C.byref(n))
        return n.value

    def choose_substeps(self, frame_dt):
        return self.L.cfo_choose_substeps(self.p, frame_dt)

    def encode_frame(self, substeps=1):
        self.L.cfo_encode_frame(self.p, substeps)

    def step_adaptive(self, dt_max):
        return self.L.cfo_step_adaptive(self.p, dt_max)

    def dry_now(self):
        self.L.cfo_dry_now(self.p)

    def host_stats(self):
        hm, hp = C.c_float(), C.c_float()
        self.L.cfo_host_stats(self.p, C.byref(hm), C.byref(hp))
        return hm.value, hp.value

    total_deposited = 0.0

    def upload_deposits(self, deps):
        """Film::upload_deposits: bins the records (deposit_ref.DEPOSIT_DTYPE)
        for the next frame; returns the number taken."""
        import deposit_ref as dr
        deps = np.ascontiguousarray(np.asarray(deps, dr.DEPOSIT_DTYPE).reshape(-1))
        hm, hp = self.host_stats()
        sent, start, cnt, items, self.total_deposited, hp = dr.bin_deposits(
            deps, self.w, self.h, self.settings.width_m, self.settings.height_m, hm, hp, self.total_deposited)
        u = C.POINTER(C.c_uint32)
        items = np.ascontiguousarray(items, np.uint32)
        self.L.cfo_set_deposits(self.p, deps.ctypes.data if sent else None, sent, start.ctypes.data_as(u),
                                cnt.ctypes.data_as(u), start.size, items.ctypes.data_as(u), items.size, hp)
        return sent

    def run(self, kernel):
        assert self.L.cfo_run(self.p, kernel.encode()), kernel

    def stats(self):
        hm, mm, a, ms = C.c_float(), C.c_float(), C.c_uint32(), C.c_double()
        self.L.cfo_stats(self.p, C.byref(hm), C.byref(mm), C.byref(a), C.byref(ms))
        return dict(h_max=hm.value, mu_min=mm.value, active_tiles=a.value, mass=ms.value)


_ref = None


def ref_lib():
    """The translated reference shaders (present only where the reference is)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            return None
        L = C.CDLL(str(REF_LIB))
        L.wgr_create.argtypes = [C.c_uint32, C.c_uint32]
        L.wgr_set_params.argtypes = [C.POINTER(Params)]
        L.wgr_set_tables.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.wgr_encode_frame.argtypes = [C.c_uint32]
        L.wgr_run.argtypes = [C.c_char_p]
        L.wgr_run.restype = C.c_int
        u32p = C.POINTER(C.c_uint32)
        L.wgr_set_deposits.argtypes = [C.c_void_p, C.c_uint32, u32p, u32p, C.c_uint32, u32p, C.c_uint32]
        L.wgr_set_implicit.argtypes = [C.c_uint32, C.c_uint32]
        L.wgr_buffer.argtypes = [C.c_char_p, C.POINTER(C.c_double), C.c_int]
        L.wgr_buffer.restype = C.c_int
        L.wgr_active_count.restype = C.c_uint32
        _ref = L
    return _ref


class RefShaders:
    """The reference WGSL, translated to C++ (FP64), one film per process."""

    def __init__(self, w, h):
        self.L = ref_lib()
        assert self.L is not None, "translated reference not built"
        self.w, self.h, self.n = w, h, w * h
        self.L.wgr_create(w, h)
        self.tiles = ((w + 15) // 16) * ((h + 15) // 16)

    def set_params(self, p):
        self.L.wgr_set_params(C.byref(p))

    def set_tables(self, pigtab, cmf):
        a, pa = _f32p(pigtab)
        b, pb = _f32p(cmf)
        self.L.wgr_set_tables(pa, pb)

    def _len(self, name):
        if name in ("tile_flags", "tile_moved"):
            return self.tiles
        if name == "stats":
            return 2 * ((self.w + 63) // 64) * ((self.h + 63) // 64)
        return PLANES[name] * self.n

    def buf(self, name):
        out = np.zeros(self._len(name), np.float64)
        assert self.L.wgr_buffer(name.encode(), out.ctypes.data_as(C.POINTER(C.c_double)), 0), name
        return out

    def set_buf(self, name, values):
        v = np.ascontiguousarray(np.asarray(values, np.float64).reshape(-1))
        assert v.size == self._len(name), (name, v.size)
        assert self.L.wgr_buffer(name.encode(), v.ctypes.data_as(C.POINTER(C.c_double)), 1), name

    def write_state(self, planes):
        for k in STATE:
            v = np.asarray(planes[k])
            if k == "rheo":
                r = np.zeros((self.n, 3))
                r[:, :2] = v.reshape(self.n, 2)
                v = r
            self.set_buf(k, v)
        self.L.wgr_after_write_state()

    def encode_frame(self, substeps=1):
        self.L.wgr_encode_frame(substeps)

    def run(self, kernel):
        assert self.L.wgr_run(kernel.encode()), kernel

    def set_implicit(self, steps, iters):
        """Film::implicit_steps and FilmSettings::implicit_iters for the next frames."""
        self.L.wgr_set_implicit(steps, iters)

    def set_deposits(self, deps, start, cnt, items):
        """Deposits for the next frame with tile tables from the
        upload_deposits restatement (deposit_ref.bin_deposits)."""
        import deposit_ref as dr
        deps = np.ascontiguousarray(np.asarray(deps, dr.DEPOSIT_DTYPE).reshape(-1))
        u = C.POINTER(C.c_uint32)
        start, cnt, items = (np.ascontiguousarray(a, np.uint32) for a in (start, cnt, items))
        self.L.wgr_set_deposits(deps.ctypes.data if deps.size else None, deps.size, start.ctypes.data_as(u),
                                cnt.ctypes.data_as(u), start.size, items.ctypes.data_as(u), items.size)


def make_settings(overrides):
    return Settings.default(**overrides)


def pack_params(settings, w, h, frame_dt, substeps, h_max=0.0, mu_min=1.0):
    """The oracle's update_params packing for explicit host stats."""
    L = lib()
    L.cfo_pack_params.argtypes = [C.POINTER(Settings), C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, C.c_float,
                                  C.c_float, C.POINTER(Params), C.POINTER(C.c_uint32)]
    p, n = Params(), C.c_uint32()
    L.cfo_pack_params(C.byref(settings), w, h, frame_dt, substeps, h_max, mu_min, C.byref(p), C.byref(n))
    return p, n.value
