"""Deposits: paint laid on a film (src/film/mod.rs:25-186).

The constructors run in the CUDA library's host code (cf_deposit_ribbon /
capsule / stroke), so a record built here is the record the reference builds,
bit for bit.  Records are numpy structured scalars/arrays of DEPOSIT_DTYPE
(the reference's 96-byte layout); Film.upload_deposits takes an array of them.
"""
import ctypes as C

import numpy as np

from . import capi

RECYCLED, CAP_START, CAP_END, METHOD_SHIFT = 1, 2, 4, 8
METHODS = {"thread": 1, "drop": 2, "pour": 3, "brush": 4, "knife": 5, "roller": 6}  # src/film/mod.rs:45-53

DEPOSIT_DTYPE = np.dtype([("p0", "<f4", 2), ("p1", "<f4", 2), ("n0", "<f4", 2), ("n1", "<f4", 2),
                          ("r0", "<f4"), ("r1", "<f4"), ("h0", "<f4"), ("vol", "<f4"),
                          ("kind", "<u4"), ("pad", "<u4", 3), ("pig", "<u4", 8)])
assert DEPOSIT_DTYPE.itemsize == C.sizeof(capi.Deposit)


def _v2(p):
    return (C.c_float * 2)(float(p[0]), float(p[1]))


def _pig(pig):
    a = np.asarray(pig, np.uint32).reshape(8)
    return (C.c_uint32 * 8)(*[int(x) for x in a])


def _record(d):
    return np.frombuffer(bytes(d), DEPOSIT_DTYPE)[0].copy()


def _check(st, what):
    if st != capi.CF_OK:
        raise capi.FilmError(st, what)


def pack_pig(values):
    """16 pigment slots -> 8 u32 words of f16 pairs (WGSL pack2x16float)."""
    v = np.asarray(values, np.float16).reshape(8, 2).view(np.uint16).astype(np.uint32)
    return (v[:, 0] | (v[:, 1] << 16)).astype(np.uint32)


def ribbon(p0, p1, n0, n1, r0, r1, caps, volume, pig, dx):
    """Deposit::ribbon: segment p0 -> p1 cut by the end normals n0, n1."""
    L = capi.load_library()
    d = capi.Deposit()
    _check(L.cf_deposit_ribbon(_v2(p0), _v2(p1), _v2(n0), _v2(n1), r0, r1, caps, volume, _pig(pig), dx,
                               C.byref(d)), "cf_deposit_ribbon")
    return _record(d)


def capsule(p0, p1, r, volume, pig, dx):
    """Deposit::capsule: a segment with round caps."""
    L = capi.load_library()
    d = capi.Deposit()
    _check(L.cf_deposit_capsule(_v2(p0), _v2(p1), r, volume, _pig(pig), dx, C.byref(d)), "cf_deposit_capsule")
    return _record(d)


def stroke(p0, p1, r, volume, pig, dx):
    """Deposit::stroke: a capsule when short, else a ribbon with square ends."""
    L = capi.load_library()
    d = capi.Deposit()
    _check(L.cf_deposit_stroke(_v2(p0), _v2(p1), r, volume, _pig(pig), dx, C.byref(d)), "cf_deposit_stroke")
    return _record(d)


def _as_struct(rec):
    return capi.Deposit.from_buffer_copy(np.asarray(rec, DEPOSIT_DTYPE).tobytes())


def sampled_volume(rec, lattice):
    """Deposit::sampled_volume: the profile summed on a lattice (m^3)."""
    out = C.c_float()
    _check(capi.load_library().cf_deposit_sampled_volume(C.byref(_as_struct(rec)), lattice, C.byref(out)),
           "cf_deposit_sampled_volume")
    return np.float32(out.value)


def height_at(rec, p):
    """The deposit's profile height at the point p (metres)."""
    out = C.c_float()
    _check(capi.load_library().cf_deposit_height_at(C.byref(_as_struct(rec)), _v2(p), C.byref(out)),
           "cf_deposit_height_at")
    return np.float32(out.value)
