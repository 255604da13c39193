"""ctypes mirror of include/canvaz_film.h (structs, enums, library loading).

This is plumbing for Python callers (tests, bench, serving loop); the product
is the CUDA library libcanvaz_film.so built from ../csrc.  Loading fails
loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR.parent / "csrc" / "_build" / "libcanvaz_film.so"

CF_OK = 0
CF_ERR_INVALID_ARG = 1
CF_ERR_OUT_OF_MEMORY = 2
CF_ERR_CUDA = 3
CF_ERR_TIMEOUT = 4
CF_ERR_NAN = 5
CF_ERR_UNSUPPORTED = 6
CF_ERR_NOT_READY = 7

CF_PREC_REFERENCE = 0
CF_PREC_FP32 = 1
CF_PREC_BF16 = 2

CF_PIG_F16 = 0
CF_PIG_F32 = 1
CF_PIG_BF16 = 2

PREC_TO_PIG = {CF_PREC_REFERENCE: CF_PIG_F16, CF_PREC_FP32: CF_PIG_F32, CF_PREC_BF16: CF_PIG_BF16}


class Settings(C.Structure):
    """cf_settings: FilmSettings (src/film/mod.rs:281-350) + env toggles."""
    _fields_ = [
        ("width_m", C.c_float), ("height_m", C.c_float), ("rho", C.c_float), ("sigma", C.c_float),
        ("n_index", C.c_float), ("m_cap", C.c_float), ("contact_angle_deg", C.c_float),
        ("hysteresis_deg", C.c_float), ("h_star", C.c_float), ("raw_canvas", C.c_int32),
        ("weave_um", C.c_float), ("cure_rate", C.c_float), ("tau_cure", C.c_float),
        ("lnmu_cure", C.c_float), ("v_cap", C.c_float), ("tilt_deg", C.c_float),
        ("tilt_dir_deg", C.c_float), ("gravity", C.c_float), ("medium_mu", C.c_float),
        ("debug_view", C.c_uint32), ("h_min", C.c_float), ("m_cap_hydro", C.c_float),
        ("max_substeps", C.c_uint32), ("min_substeps", C.c_uint32), ("implicit_iters", C.c_uint32),
        ("implicit_hydro", C.c_int32), ("slump", C.c_int32), ("capillary", C.c_int32),
        ("capillary_implicit", C.c_int32), ("no_hold", C.c_int32), ("no_transl", C.c_int32),
        ("no_shape", C.c_int32), ("no_cap", C.c_int32), ("kshape", C.c_float), ("kline", C.c_float),
        ("hyst_deg", C.c_float), ("fcap_exp", C.c_float), ("cap_cond", C.c_float),
        ("all_active", C.c_int32),
    ]

    @classmethod
    def default(cls, **kw):
        """FilmSettings::default (src/film/mod.rs:315-350), then overrides."""
        s = cls(
            width_m=1.2, height_m=0.8, rho=1000.0, sigma=0.035, n_index=1.0, m_cap=1.0e-8,
            contact_angle_deg=45.0, hysteresis_deg=15.0, h_star=2.0e-5, raw_canvas=1, weave_um=25.0,
            cure_rate=1.0 / 600.0, tau_cure=300.0, lnmu_cure=5.0, v_cap=1.0, tilt_deg=0.0,
            tilt_dir_deg=-90.0, gravity=9.81, medium_mu=0.08, debug_view=0, h_min=1.5e-5,
            m_cap_hydro=1.0e-7, max_substeps=64, min_substeps=4, implicit_iters=40, implicit_hydro=1,
            slump=0, capillary=1, capillary_implicit=0, no_hold=0, no_transl=0, no_shape=0, no_cap=0,
            kshape=1.0, kline=0.0, hyst_deg=-1.0, fcap_exp=2.5, cap_cond=80.0, all_active=0,
        )
        for k, v in kw.items():
            if not hasattr(s, k):
                raise AttributeError(k)
            setattr(s, k, v)
        return s

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Params(C.Structure):
    """cf_params: the Params uniform (src/film/mod.rs:5-23), 176 bytes."""
    _fields_ = [
        ("size", C.c_uint32 * 2), ("tiles", C.c_uint32 * 2), ("dx", C.c_float), ("dt", C.c_float),
        ("inv_dx", C.c_float), ("frame_dt", C.c_float), ("g", C.c_float * 4), ("phys", C.c_float * 4),
        ("ein", C.c_float * 4), ("cure", C.c_float * 4), ("misc", C.c_float * 4),
        ("flags", C.c_uint32 * 4), ("front", C.c_float * 4), ("front2", C.c_float * 4),
        ("front3", C.c_float * 4),
    ]

    def raw(self):
        return bytes(self)


class StateView(C.Structure):
    """cf_state_view: the eight persistent planes (src/film/mod.rs:1277-1279)."""
    _fields_ = [
        ("h", C.c_void_p), ("m", C.c_void_p), ("rheo", C.c_void_p), ("strata_h", C.c_void_p),
        ("strata_pig", C.c_void_p), ("strata_cure", C.c_void_p), ("sub_refl", C.c_void_p),
        ("lay", C.c_void_p), ("pig_format", C.c_int32), ("device", C.c_int32),
    ]


class ResolveParams(C.Structure):
    """cf_resolve_params (the Res uniform of shaders/resolve.wgsl)."""
    _fields_ = [("scale", C.c_float), ("exposure_ev", C.c_float), ("bloom", C.c_float), ("grain", C.c_float),
                ("vignette", C.c_float), ("sharpen", C.c_float), ("agx", C.c_int32), ("reserved", C.c_int32)]


class SnapshotInfo(C.Structure):
    """cf_snapshot_info: the painting-file header fields (src/session.rs:248-310)."""
    _fields_ = [("w", C.c_uint32), ("h", C.c_uint32), ("tilt_deg", C.c_float), ("tilt_dir_deg", C.c_float),
                ("cure_rate", C.c_float), ("h_max", C.c_float), ("s_max", C.c_float), ("total_deposited", C.c_double)]


class Deposit(C.Structure):
    """cf_deposit: Deposit (src/film/mod.rs:25-39), 96 bytes."""
    _fields_ = [("p0", C.c_float * 2), ("p1", C.c_float * 2), ("n0", C.c_float * 2), ("n1", C.c_float * 2),
                ("r0", C.c_float), ("r1", C.c_float), ("h0", C.c_float), ("vol", C.c_float),
                ("kind", C.c_uint32), ("pad", C.c_uint32 * 3), ("pig", C.c_uint32 * 8)]


assert C.sizeof(Deposit) == 96
CF_MAX_DEPOSITS = 65536


class ReliefView(C.Structure):
    """cf_relief_view."""
    _fields_ = [("x0", C.c_float), ("y0", C.c_float), ("pixel_m", C.c_float), ("width", C.c_uint32),
                ("height", C.c_uint32), ("light", C.c_float * 3), ("ambient", C.c_float), ("reserved", C.c_uint32)]


class RenderCam(C.Structure):
    """cf_render_cam: the renderer's camera uniform (76 words, render.wgsl:1-15)."""
    _fields_ = [("inv_vp", C.c_float * 16), ("eye", C.c_float * 4), ("canvas", C.c_float * 4), ("light", C.c_float * 4),
                ("size", C.c_uint32 * 4), ("sky", C.c_float * 4), ("ground", C.c_float * 4), ("vp", C.c_float * 16),
                ("jitter", C.c_float * 4), ("ortho", C.c_float * 4), ("basis_r", C.c_float * 4),
                ("basis_u", C.c_float * 4), ("lens", C.c_float * 4)]

    @classmethod
    def from_words(cls, words):
        """From the uniform's 76 32-bit words (float32 array; size as u32 bit patterns)."""
        import numpy as np
        w = np.ascontiguousarray(np.asarray(words, np.float32))
        assert w.size == 76
        return cls.from_buffer_copy(w.tobytes())


class BatchTuning(C.Structure):
    """cf_batch_tuning."""
    _fields_ = [("list_blocks_per_sm", C.c_uint32), ("use_graph", C.c_uint32), ("frames_per_graph", C.c_uint32),
                ("tiles_per_block", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [
        ("h_max", C.c_float), ("mu_min", C.c_float), ("active_tiles", C.c_uint32),
        ("frames", C.c_uint32), ("wet_volume", C.c_double), ("relief_volume", C.c_double),
        ("last_dt", C.c_double), ("nan_cells", C.c_uint64), ("wet_cells", C.c_uint64),
        ("launches", C.c_uint64),
    ]


assert C.sizeof(Params) == 176


class FilmError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("cf status %d: %s" % (status, msg))
        self.status = status


_lib = None


def load_library(path=None):
    """Loads the CUDA product library (built by build.py).  Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path or os.environ.get("CANVAZ_FILM_LIB", LIB_PATH))
    if not p.exists():
        raise FileNotFoundError("CUDA film library not built: %s (run __graft_entry__.build())" % p)
    lib = C.CDLL(str(p))
    vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int32, C.c_float
    sig = {
        "cf_settings_default": ([C.POINTER(Settings)], i32),
        "cf_create": ([C.POINTER(Settings), u32, u32, i32, C.POINTER(vp)], i32),
        "cf_destroy": ([vp], i32),
        "cf_set_tables": ([vp, C.POINTER(f32), C.POINTER(f32)], i32),
        "cf_write_state": ([vp, C.POINTER(StateView)], i32),
        "cf_read_state": ([vp, C.POINTER(StateView)], i32),
        "cf_update_params": ([vp, f32, u32], i32),
        "cf_choose_substeps": ([vp, f32, C.POINTER(u32)], i32),
        "cf_encode_frame": ([vp, u32, vp], i32),
        "cf_step_adaptive": ([vp, f32, vp], i32),
        "cf_dry_now": ([vp, vp], i32),
        "cf_color_device_ptr": ([vp, C.POINTER(vp)], i32),
        "cf_read_color": ([vp, C.POINTER(C.c_uint16)], i32),
        "cf_write_state_async": ([vp, C.POINTER(StateView), vp], i32),
        "cf_read_state_async": ([vp, C.POINTER(StateView), vp], i32),
        "cf_read_color_async": ([vp, C.POINTER(C.c_uint16), vp], i32),
        "cf_get_stats": ([vp, C.POINTER(Stats)], i32),
        "cf_get_params": ([vp, C.POINTER(Params)], i32),
        "cf_sync": ([vp], i32),
        "cf_last_error": ([vp], C.c_char_p),
        "cf_cfl_stats_noalloc": ([vp, vp, u32, u32, f32, vp, vp], i32),
        "cf_film_bytes": ([u32, u32, i32, C.POINTER(C.c_uint64)], i32),
        "cf_clone_state": ([vp, vp, vp], i32),
        "cf_resolve": ([vp, C.POINTER(ResolveParams), vp, vp], i32),
        "cf_snapshot_save": ([vp, C.POINTER(SnapshotInfo), C.POINTER(C.POINTER(C.c_uint8)), C.POINTER(C.c_uint64)], i32),
        "cf_snapshot_free": ([C.POINTER(C.c_uint8)], i32),
        "cf_snapshot_load": ([vp, C.c_char_p, C.c_uint64, C.POINTER(SnapshotInfo)], i32),
        "cf_lz4_compress": ([C.c_char_p, C.c_uint64, vp, C.c_uint64, C.POINTER(C.c_uint64)], i32),
        "cf_lz4_decompress": ([C.c_char_p, C.c_uint64, vp, C.c_uint64, C.POINTER(C.c_uint64)], i32),
        "cf_deposit_ribbon": ([C.POINTER(f32), C.POINTER(f32), C.POINTER(f32), C.POINTER(f32), f32, f32, u32, f32,
                               C.POINTER(u32), f32, C.POINTER(Deposit)], i32),
        "cf_deposit_capsule": ([C.POINTER(f32), C.POINTER(f32), f32, f32, C.POINTER(u32), f32, C.POINTER(Deposit)],
                               i32),
        "cf_deposit_stroke": ([C.POINTER(f32), C.POINTER(f32), f32, f32, C.POINTER(u32), f32, C.POINTER(Deposit)],
                              i32),
        "cf_deposit_sampled_volume": ([C.POINTER(Deposit), f32, C.POINTER(f32)], i32),
        "cf_deposit_height_at": ([C.POINTER(Deposit), C.POINTER(f32), C.POINTER(f32)], i32),
        "cf_upload_deposits": ([vp, vp, u32, C.POINTER(u32), C.POINTER(C.c_double)], i32),
        "cf_lay_deposits": ([vp, vp], i32),
        "cf_sample_relief": ([vp, vp, u32, vp, vp], i32),
        "cf_relief_shadow": ([vp, vp, u32, C.POINTER(f32), f32, vp, vp], i32),
        "cf_render_relief": ([vp, C.POINTER(ReliefView), vp, vp], i32),
        "cf_render_lit": ([vp, C.POINTER(RenderCam), C.c_uint32, C.c_uint32, vp, vp, vp], i32),
        "cf_batch_create": ([C.POINTER(vp)], i32),
        "cf_batch_destroy": ([vp], i32),
        "cf_batch_add": ([vp, vp], i32),
        "cf_batch_remove": ([vp, vp], i32),
        "cf_batch_info": ([vp, C.POINTER(u32), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], i32),
        "cf_batch_set_tuning": ([vp, C.POINTER(BatchTuning)], i32),
        "cf_batch_get_tuning": ([vp, C.POINTER(BatchTuning)], i32),
        "cf_batch_step": ([vp, u32, u32, f32, vp], i32),
        "cf_batch_autotune": ([vp, u32, u32, f32, vp, C.POINTER(BatchTuning), C.POINTER(f32)], i32),
        "cf_batch_last_error": ([vp], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def header_symbols(header=None):
    """Names of the functions declared in an include/*.h header."""
    import re
    h = Path(header) if header else PKG_DIR.parent.parent / "include" / "canvaz_film.h"
    txt = h.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cf\w+)\s*\(", txt)))


def film_bytes(w, h, precision):
    """cf_film_bytes: device bytes of a w x h film (admission budgeting)."""
    out = C.c_uint64()
    st = load_library().cf_film_bytes(w, h, precision, C.byref(out))
    if st != CF_OK:
        raise FilmError(st, "cf_film_bytes")
    return out.value
