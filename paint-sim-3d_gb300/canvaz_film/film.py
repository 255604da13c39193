"""Python host mirror of the reference's `impl Film` over the C ABI.

Method names, argument meaning and order follow src/film/mod.rs (Film::new,
update_params, choose_substeps, encode_frame, write_state, read_state,
dry_now).  Every call goes through libcanvaz_film.so (the sm_103a kernels);
a missing library or device raises: there is no CPU fallback.
"""
import ctypes as C

import numpy as np

from . import capi
from .capi import BatchTuning, FilmError, Params, Settings, SnapshotInfo, StateView, Stats

_f32p = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731

# Elements per cell of the debug planes (include/canvaz_film_debug.h)
DEBUG_PER_CELL = {
    "h": 1, "m": 1, "mu": 1, "tau": 1, "nn": 1, "delta": 1, "lay": 1, "pres": 2, "fnorm": 2, "flux": 4, "acc": 4,
    "acc_s": 16, "alpha_s": 4, "alpha": 1, "tmp": 1, "h_frame": 1, "strata_h": 4, "strata_cure": 4,
    "strata_h2": 4, "strata_cure2": 4, "strata_pig": 64, "strata_pig2": 64, "sub_refl": 16, "color": 4,
    "fill_src": 1, "fflags": 1, "h_next": 1, "delta_old": 1, "detail": 4,
}
_ELEM_DTYPE = {0: np.float32, 1: np.uint32, 2: np.float16, 3: "bf16", 4: np.int32}


def _bf16_to_f32(u16):
    return (u16.astype(np.uint32) << 16).view(np.float32)


def _f32_to_bf16(x):
    """Round-to-nearest-even f32 -> bf16 bits."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def _pig_to_bf16(x):
    """Pigment slots (16 per stratum, last axis a multiple of 16) as the BF16
    format's bits: slot 14, the viscosity override ln mu + 10 (0 = none), is
    stored as mu itself (Pa s); every other slot as its value."""
    a = np.array(x, np.float32)
    v = a.reshape(-1, 16)
    s14 = v[:, 14].astype(np.float64)
    v[:, 14] = np.where(s14 > 0, np.exp(np.where(s14 > 0, s14, 10.0) - 10.0), 0.0).astype(np.float32)
    return _f32_to_bf16(a)


def _pig_from_bf16(u16):
    """The inverse of _pig_to_bf16: slot values as float32 (slot 14 back to
    ln mu + 10, 0 where no override is stored)."""
    u = np.asarray(u16, np.uint16)
    a = _bf16_to_f32(u).copy()
    v = a.reshape(-1, 16)
    b = u.reshape(-1, 16)[:, 14]
    mu = np.where(b != 0, v[:, 14], np.float32(1.0)).astype(np.float32)
    v[:, 14] = np.where(b != 0, np.log(mu) + np.float32(10.0), np.float32(0.0)).astype(np.float32)
    return a


_PIG_PLANES = ("strata_pig", "strata_pig2")


def _lib():
    L = capi.load_library()
    if not hasattr(L, "_debug_bound"):
        vp, i32 = C.c_void_p, C.c_int32
        for name, args in {
            "cf_debug_plane_info": [vp, C.c_char_p, C.POINTER(C.c_size_t), C.POINTER(i32)],
            "cf_debug_read": [vp, C.c_char_p, vp, C.c_size_t],
            "cf_debug_write": [vp, C.c_char_p, vp, C.c_size_t],
            "cf_debug_run": [vp, C.c_char_p, vp],
            "cf_debug_set_params": [vp, C.POINTER(Params)],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = i32
        L.cf_pack_params.argtypes = [C.POINTER(Settings), C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, C.c_float,
                                     C.c_float, C.POINTER(Params), C.POINTER(C.c_uint32)]
        L.cf_pack_params.restype = i32
        L._debug_bound = True
    return L


def pack_params(settings, w, h, frame_dt, substeps, h_max=0.0, mu_min=1.0):
    """cf_pack_params: update_params' packing, host only."""
    L = _lib()
    p, n = Params(), C.c_uint32()
    st = L.cf_pack_params(C.byref(settings), w, h, frame_dt, substeps, h_max, mu_min, C.byref(p), C.byref(n))
    if st != capi.CF_OK:
        raise FilmError(st, "cf_pack_params")
    return p, n.value


class Film:
    """One canvas on the GPU (Film::new, src/film/mod.rs:578)."""

    def __init__(self, settings, w, h, precision=capi.CF_PREC_REFERENCE):
        self.L = _lib()
        self.w, self.h, self.n = w, h, w * h
        self.settings = settings
        self.precision = precision
        self.p = C.c_void_p()
        st = self.L.cf_create(C.byref(settings), w, h, precision, C.byref(self.p))
        if st != capi.CF_OK:
            raise FilmError(st, self.L.cf_last_error(None).decode())

    def _check(self, st, what):
        if st != capi.CF_OK:
            raise FilmError(st, "%s: %s" % (what, self.L.cf_last_error(self.p).decode()))

    def close(self):
        if self.p:
            self.L.cf_destroy(self.p)
            self.p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tables(self, pigtab, cmf):
        a = np.ascontiguousarray(pigtab, np.float32)
        b = np.ascontiguousarray(cmf, np.float32)
        self._check(self.L.cf_set_tables(self.p, _f32p(a), _f32p(b)), "cf_set_tables")

    def write_state(self, planes, pig_format=None):
        """Film::write_state: planes is a dict of numpy arrays (oracle layout);
        strata_pig values are converted to `pig_format` (default: the film's)."""
        fmt = capi.PREC_TO_PIG[self.precision] if pig_format is None else pig_format
        keep = {}
        v = StateView(pig_format=fmt, device=0)
        for k, dt in (("h", np.float32), ("m", np.float32), ("rheo", np.float32), ("strata_h", np.float32),
                      ("strata_cure", np.float32), ("lay", np.uint32)):
            if k in planes:
                a = np.ascontiguousarray(planes[k], dt)
                keep[k] = a
                setattr(v, k, a.ctypes.data)
        if "sub_refl" in planes:
            a = np.ascontiguousarray(planes["sub_refl"], np.float32).astype(np.float16)
            keep["sub_refl"] = a
            v.sub_refl = a.ctypes.data
        if "strata_pig" in planes:
            x = np.ascontiguousarray(planes["strata_pig"], np.float32)
            if fmt == capi.CF_PIG_F32:
                a = x
            elif fmt == capi.CF_PIG_F16:
                a = x.astype(np.float16)
            else:
                a = _pig_to_bf16(x)
            a = np.ascontiguousarray(a)
            keep["strata_pig"] = a
            v.strata_pig = a.ctypes.data
        self._check(self.L.cf_write_state(self.p, C.byref(v)), "cf_write_state")

    def read_state(self, pig_format=capi.CF_PIG_F32):
        """Film::read_state as a dict of numpy arrays (pigments as float32)."""
        n = self.n
        out = {"h": np.zeros(n, np.float32), "m": np.zeros(n, np.float32), "rheo": np.zeros((n, 2), np.float32),
               "strata_h": np.zeros((n, 4), np.float32), "strata_cure": np.zeros((n, 4), np.float32),
               "sub_refl": np.zeros((n, 16), np.float16), "lay": np.zeros(n, np.uint32)}
        pig = np.zeros((n, 64), np.float32 if pig_format == capi.CF_PIG_F32 else np.uint16)
        v = StateView(pig_format=pig_format, device=0)
        for k, a in out.items():
            setattr(v, k, a.ctypes.data)
        v.strata_pig = pig.ctypes.data
        self._check(self.L.cf_read_state(self.p, C.byref(v)), "cf_read_state")
        if pig_format == capi.CF_PIG_F16:
            pig = pig.view(np.float16).astype(np.float32)
        elif pig_format == capi.CF_PIG_BF16:
            pig = _pig_from_bf16(pig)
        out["strata_pig"] = pig
        out["sub_refl"] = out["sub_refl"].astype(np.float32)
        return out

    def clone_from(self, src, stream=None):
        """cf_clone_state: src's whole device state into this film (same size
        and precision), stream-ordered, no host round trip."""
        self._check(self.L.cf_clone_state(self.p, src.p, stream), "cf_clone_state")

    def save_snapshot(self, **header):
        """App::save_painting's bytes (cf_snapshot_save); header fields:
        tilt_deg, tilt_dir_deg, cure_rate, h_max, s_max, total_deposited."""
        info = SnapshotInfo(w=self.w, h=self.h, tilt_deg=self.settings.tilt_deg,
                            tilt_dir_deg=self.settings.tilt_dir_deg, cure_rate=self.settings.cure_rate)
        for k, v in header.items():
            setattr(info, k, v)
        buf, n = C.POINTER(C.c_uint8)(), C.c_uint64()
        self._check(self.L.cf_snapshot_save(self.p, C.byref(info), C.byref(buf), C.byref(n)), "cf_snapshot_save")
        try:
            return C.string_at(buf, n.value)
        finally:
            self.L.cf_snapshot_free(buf)

    def load_snapshot(self, data):
        """App::open_painting (cf_snapshot_load); returns the header fields."""
        info = SnapshotInfo()
        self._check(self.L.cf_snapshot_load(self.p, data, len(data), C.byref(info)), "cf_snapshot_load")
        return {k: getattr(info, k) for k, _ in SnapshotInfo._fields_}

    total_deposited = 0.0

    def upload_deposits(self, deps):
        """Film::upload_deposits (cf_upload_deposits): the records (an array of
        deposit.DEPOSIT_DTYPE) are laid by the next frame.  Returns the number
        taken (at most CF_MAX_DEPOSITS); the caller keeps the rest."""
        from .deposit import DEPOSIT_DTYPE
        a = np.ascontiguousarray(np.asarray(deps, DEPOSIT_DTYPE).reshape(-1))
        sent, tot = C.c_uint32(), C.c_double()
        self._check(self.L.cf_upload_deposits(self.p, a.ctypes.data if a.size else None, a.size, C.byref(sent),
                                              C.byref(tot)), "cf_upload_deposits")
        self.total_deposited = tot.value
        return sent.value

    def sample_relief(self, points_ptr, n, out_ptr, stream=None):
        """cf_sample_relief: 8 floats per canvas point (device pointers)."""
        self._check(self.L.cf_sample_relief(self.p, points_ptr, n, out_ptr, stream), "cf_sample_relief")

    def relief_shadow(self, points_ptr, n, light, top, out_ptr, stream=None):
        """cf_relief_shadow: per (x, y, z0) point, surf_bilinear and the key
        light's shadow factor (device pointers)."""
        lt = (C.c_float * 3)(*light)
        self._check(self.L.cf_relief_shadow(self.p, points_ptr, n, lt, top, out_ptr, stream), "cf_relief_shadow")

    def render_relief(self, out_ptr, x0, y0, pixel_m, width, height, light=(0.3, 0.5, 0.8), ambient=0.35,
                      stream=None):
        """cf_render_relief: a width x height RGBA8 top-down view into out_ptr (device)."""
        v = capi.ReliefView(x0=x0, y0=y0, pixel_m=pixel_m, width=width, height=height, ambient=ambient)
        for k in range(3):
            v.light[k] = light[k]
        self._check(self.L.cf_render_relief(self.p, C.byref(v), out_ptr, stream), "cf_render_relief")

    def render_lit(self, cam, width, height, out_f32_ptr=None, out_rgba8_ptr=None, stream=None):
        """cf_render_lit: the renderer's fragment shader over the film for a
        width x height target, into device buffers (RGBA floats and/or RGBA8).
        `cam` is a capi.RenderCam or the uniform's 76 words."""
        if not isinstance(cam, capi.RenderCam):
            cam = capi.RenderCam.from_words(cam)
        self._check(self.L.cf_render_lit(self.p, C.byref(cam), width, height, out_f32_ptr, out_rgba8_ptr, stream),
                    "cf_render_lit")

    def lay_deposits(self, stream=None):
        """cf_lay_deposits: lays the uploaded deposits now (asynchronous)."""
        self._check(self.L.cf_lay_deposits(self.p, stream), "cf_lay_deposits")

    def update_params(self, frame_dt, substeps):
        self._check(self.L.cf_update_params(self.p, frame_dt, substeps), "cf_update_params")

    def choose_substeps(self, frame_dt):
        n = C.c_uint32()
        self._check(self.L.cf_choose_substeps(self.p, frame_dt, C.byref(n)), "cf_choose_substeps")
        return n.value

    def encode_frame(self, substeps=1, stream=None):
        self._check(self.L.cf_encode_frame(self.p, substeps, stream), "cf_encode_frame")

    def step_adaptive(self, dt_max, stream=None):
        self._check(self.L.cf_step_adaptive(self.p, dt_max, stream), "cf_step_adaptive")

    def dry_now(self, stream=None):
        self._check(self.L.cf_dry_now(self.p, stream), "cf_dry_now")

    def sync(self):
        self._check(self.L.cf_sync(self.p), "cf_sync")

    def params(self):
        p = Params()
        self._check(self.L.cf_get_params(self.p, C.byref(p)), "cf_get_params")
        return p

    def set_params(self, p):
        self._check(self.L.cf_debug_set_params(self.p, C.byref(p)), "cf_debug_set_params")

    def stats(self):
        s = Stats()
        self._check(self.L.cf_get_stats(self.p, C.byref(s)), "cf_get_stats")
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def color(self):
        """color_tex as float32 (n, 4): linear sRGB + roughness (rgba16f)."""
        out = np.zeros((self.n, 4), np.uint16)
        self._check(self.L.cf_read_color(self.p, out.ctypes.data_as(C.POINTER(C.c_uint16))), "cf_read_color")
        return out.view(np.float16).astype(np.float32)

    def resolve(self, out_ptr, stream=None, **params):
        """cf_resolve: the display epilogue of the colour plane into a device
        buffer of w x h RGBA8 pixels at out_ptr."""
        p = capi.ResolveParams(scale=1.0, exposure_ev=0.0, bloom=0.0, grain=0.0, vignette=0.0, sharpen=0.0, agx=1)
        for k, v in params.items():
            setattr(p, k, v)
        self._check(self.L.cf_resolve(self.p, C.byref(p), out_ptr, stream), "cf_resolve")

    def color_device_ptr(self):
        p = C.c_void_p()
        self._check(self.L.cf_color_device_ptr(self.p, C.byref(p)), "cf_color_device_ptr")
        return p.value

    # ---- inspection (include/canvaz_film_debug.h) ----
    def plane(self, name):
        """A named device plane as float64/uint32 values (pig/rheo converted)."""
        nb, el = C.c_size_t(), C.c_int32()
        self._check(self.L.cf_debug_plane_info(self.p, name.encode(), C.byref(nb), C.byref(el)), name)
        dt = _ELEM_DTYPE[el.value]
        raw = np.zeros(nb.value, np.uint8)
        self._check(self.L.cf_debug_read(self.p, name.encode(), raw.ctypes.data, nb.value), name)
        if dt == "bf16":
            conv = _pig_from_bf16 if name in _PIG_PLANES else _bf16_to_f32
            return conv(raw.view(np.uint16)).astype(np.float64)
        a = raw.view(dt)
        return a.astype(np.uint64) if dt in (np.uint32,) else a.astype(np.float64)

    def set_plane(self, name, values):
        nb, el = C.c_size_t(), C.c_int32()
        self._check(self.L.cf_debug_plane_info(self.p, name.encode(), C.byref(nb), C.byref(el)), name)
        dt = _ELEM_DTYPE[el.value]
        v = np.asarray(values).reshape(-1)
        if dt == "bf16":
            a = (_pig_to_bf16 if name in _PIG_PLANES else _f32_to_bf16)(v.astype(np.float32))
        else:
            a = np.ascontiguousarray(v.astype(dt))
        assert a.nbytes == nb.value, (name, a.nbytes, nb.value)
        self._check(self.L.cf_debug_write(self.p, name.encode(), a.ctypes.data, a.nbytes), name)

    def run(self, kernel, stream=None):
        self._check(self.L.cf_debug_run(self.p, kernel.encode(), stream), kernel)


class Batch:
    """Many films stepped together (cf_batch_*): one launch per dispatch over
    every film's tiles, optionally replayed from captured CUDA graphs.  Each
    film's result equals stepping it alone with Film.encode_frame /
    Film.step_adaptive."""

    def __init__(self):
        self.L = _lib()
        self.p = C.c_void_p()
        self._check(self.L.cf_batch_create(C.byref(self.p)), "cf_batch_create")
        self.films = []

    def _check(self, st, what):
        if st != capi.CF_OK:
            msg = self.L.cf_batch_last_error(self.p).decode() if self.p else ""
            raise FilmError(st, "%s: %s" % (what, msg))

    def add(self, film):
        self._check(self.L.cf_batch_add(self.p, film.p), "cf_batch_add")
        self.films.append(film)

    def remove(self, film):
        self._check(self.L.cf_batch_remove(self.p, film.p), "cf_batch_remove")
        self.films.remove(film)

    def step(self, frames=1, substeps=1, dt_max=0.0, stream=None):
        """dt_max > 0: adaptive frames; else each film's cf_update_params
        with `substeps` substeps."""
        self._check(self.L.cf_batch_step(self.p, frames, substeps, dt_max, stream), "cf_batch_step")

    def info(self):
        nf, cells, launches = C.c_uint32(), C.c_uint64(), C.c_uint64()
        self._check(self.L.cf_batch_info(self.p, C.byref(nf), C.byref(cells), C.byref(launches)), "cf_batch_info")
        return {"films": nf.value, "cells": cells.value, "launches": launches.value}

    @property
    def tuning(self):
        t = BatchTuning()
        self._check(self.L.cf_batch_get_tuning(self.p, C.byref(t)), "cf_batch_get_tuning")
        return {k: getattr(t, k) for k, _ in BatchTuning._fields_}

    @tuning.setter
    def tuning(self, d):
        t = BatchTuning(**{**self.tuning, **d})
        self._check(self.L.cf_batch_set_tuning(self.p, C.byref(t)), "cf_batch_set_tuning")

    def autotune(self, frames_per_trial=4, substeps=1, dt_max=0.0, stream=None):
        """The project autotuner; steps the films.  Returns (tuning, ms per frame)."""
        t, ms = BatchTuning(), C.c_float()
        self._check(self.L.cf_batch_autotune(self.p, frames_per_trial, substeps, dt_max, stream, C.byref(t),
                                             C.byref(ms)), "cf_batch_autotune")
        return {k: getattr(t, k) for k, _ in BatchTuning._fields_}, ms.value

    def close(self):
        if self.p:
            self.L.cf_batch_destroy(self.p)
            self.p = C.c_void_p()
            self.films = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
