"""Asynchronous state upload and readback (cf_write_state_async,
cf_read_state_async, cf_read_color_async) against the synchronous calls:
film b gets its state from pinned host buffers asynchronously, steps on a
side stream and is read back asynchronously; film a does the same through
the synchronous calls; every plane and the colour image agree bit for bit."""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po
from canvaz_film import capi, synth

pytestmark = pytest.mark.gpu

PLANES = {"h": (1, np.float32), "m": (1, np.float32), "rheo": (2, np.float32), "strata_h": (4, np.float32),
          "strata_cure": (4, np.float32), "sub_refl": (16, np.float16), "lay": (1, np.uint32),
          "strata_pig": (64, np.float32)}


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def pinned(n, per, dt, keep):
    import torch
    t = torch.empty(n * per * np.dtype(dt).itemsize, dtype=torch.uint8).pin_memory()
    keep.append(t)
    return t.numpy().view(dt).reshape(n, per) if per > 1 else t.numpy().view(dt)


@pytest.mark.parametrize("prec", [capi.CF_PREC_REFERENCE, capi.CF_PREC_FP32, capi.CF_PREC_BF16])
def test_async_write_read_match_sync(built, prec):
    import torch
    from canvaz_film.film import Film
    cv = synth.blob_canvas(72, 56, 3, n_blobs=5, sigma=(3, 9), tables="reference")
    st = po.make_settings(cv.settings)
    a = Film(st, cv.w, cv.h, prec)
    b = Film(st, cv.w, cv.h, prec)
    for f in (a, b):
        f.set_tables(cv.pigtab, cv.cmf)
    a.write_state(cv.planes)
    src = a.read_state(pig_format=capi.CF_PIG_F32)  # f32 pigments: converted to each storage on upload
    n = cv.w * cv.h
    keep = []
    v = capi.StateView(pig_format=capi.CF_PIG_F32, device=0)
    for k, (per, dt) in PLANES.items():
        buf = pinned(n, per, dt, keep)
        buf[...] = np.asarray(src[k]).reshape(buf.shape).astype(dt)
        setattr(v, k, buf.ctypes.data)
    L = capi.load_library()
    s = torch.cuda.Stream()
    a.write_state({k: np.asarray(src[k]) for k in PLANES}, pig_format=capi.CF_PIG_F32)
    assert L.cf_write_state_async(b.p, C.byref(v), s.cuda_stream) == capi.CF_OK
    a.update_params(1e-3, 1)
    b.update_params(1e-3, 1)  # refreshes b's host stats after the asynchronous write
    assert bytes(a.params()) == bytes(b.params())
    a.encode_frame(1)
    b.encode_frame(1, s.cuda_stream)
    ov = capi.StateView(pig_format=capi.CF_PIG_F32, device=0)
    outs = {}
    for k, (per, dt) in PLANES.items():
        outs[k] = pinned(n, per, dt, keep)
        setattr(ov, k, outs[k].ctypes.data)
    col = pinned(n, 4, np.uint16, keep)
    assert L.cf_read_state_async(b.p, C.byref(ov), s.cuda_stream) == capi.CF_OK
    assert L.cf_read_color_async(b.p, col.ctypes.data_as(C.POINTER(C.c_uint16)), s.cuda_stream) == capi.CF_OK
    s.synchronize()
    want = a.read_state(pig_format=capi.CF_PIG_F32)
    for k, (per, dt) in PLANES.items():
        ref = np.asarray(want[k]).reshape(outs[k].shape).astype(dt)
        assert np.array_equal(outs[k].view(np.uint8), ref.view(np.uint8)), k
    assert np.array_equal(col.view(np.float16).astype(np.float32), a.color())


def test_async_rejects_pageable(built):
    from canvaz_film.film import Film
    cv = synth.blob_canvas(32, 32, 1, n_blobs=2, tables="reference")
    f = Film(po.make_settings(cv.settings), cv.w, cv.h, capi.CF_PREC_FP32)
    h = np.zeros(cv.w * cv.h, np.float32)
    v = capi.StateView(pig_format=capi.CF_PIG_F32, device=0, h=h.ctypes.data)
    L = capi.load_library()
    assert L.cf_write_state_async(f.p, C.byref(v), None) == capi.CF_ERR_INVALID_ARG
    assert L.cf_read_state_async(f.p, C.byref(v), None) == capi.CF_ERR_INVALID_ARG
    col = np.zeros(cv.w * cv.h * 4, np.uint16)
    assert L.cf_read_color_async(f.p, col.ctypes.data_as(C.POINTER(C.c_uint16)), None) == capi.CF_ERR_INVALID_ARG
