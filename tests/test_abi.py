"""The C-ABI library without a GPU: it builds, loads, exports every function
that include/*.h declares, and its host-side parameter packing
(update_params, src/film/mod.rs:869-917) equals the oracle's bit for bit."""
import ctypes as C
import json
import re
from pathlib import Path

import numpy as np
import pytest

import pyoracle as po
from canvaz_film import capi

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(cf_\w+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not capi.LIB_PATH.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("cf_build", ROOT / "paint-sim-3d_gb300" / "build.py")
        b = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(b)
        b.build()
    return C.CDLL(str(capi.LIB_PATH))


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_header_structs_match_ctypes():
    hdr = (ROOT / "include" / "canvaz_film.h").read_text()
    body = re.search(r"typedef struct cf_settings \{(.*?)\} cf_settings;", hdr, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"\b(?:float|int32_t|uint32_t)\s+(\w+);", body)
    assert fields == [f for f, _ in capi.Settings._fields_]
    assert C.sizeof(capi.Params) == 176


def test_settings_default_matches_reference_defaults(lib):
    lib.cf_settings_default.argtypes = [C.POINTER(capi.Settings)]
    s = capi.Settings()
    assert lib.cf_settings_default(C.byref(s)) == 0
    d = capi.Settings.default()
    o = capi.Settings()
    po.lib().cfo_settings_default.argtypes = [C.POINTER(capi.Settings)]
    po.lib().cfo_settings_default(C.byref(o))
    for k, _ in capi.Settings._fields_:
        assert getattr(s, k) == getattr(d, k) == getattr(o, k), k


CASES = [
    dict(),
    dict(tilt_deg=60.0, tilt_dir_deg=90.0, rho=1300.0, sigma=0.03, width_m=2.048, height_m=2.048),
    dict(no_hold=1, no_transl=1, no_shape=1, no_cap=1, kline=0.5, hyst_deg=5.0, capillary_implicit=1),
    dict(contact_angle_deg=70.0, n_index=0.7, debug_view=1, slump=1, implicit_hydro=0),
]


@pytest.mark.parametrize("over", CASES)
@pytest.mark.parametrize("sched", [(1 / 60, 4, 0.0, 1.0), (1e-3, 1, 3e-3, 0.5), (2e-4, 7, 1e-3, 0.05)])
def test_pack_params_bit_exact_vs_oracle(lib, over, sched):
    from canvaz_film.film import pack_params
    fdt, n, hmax, mumin = sched
    s = capi.Settings.default(**over)
    p, ni = pack_params(s, 512, 384, fdt, n, hmax, mumin)
    ref, nref = po.pack_params(s, 512, 384, fdt, n, hmax, mumin)
    assert bytes(p) == bytes(ref)
    assert ni == nref
