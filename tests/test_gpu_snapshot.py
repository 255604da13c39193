"""Painting files (cf_snapshot_save / cf_snapshot_load) on the GPU: the
bytes parse with the independent restatement of src/session.rs, hold the
eight read_state planes, and load back into a film; two films loaded from
the same file step identically."""
import numpy as np
import pytest

import lz4_ref
import pyoracle as po
from canvaz_film import capi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def stepped_film(prec):
    from canvaz_film.film import Film
    cv = synth.drip_canvas(96, 80, 5, n_lines=8)
    f = Film(po.make_settings(cv.settings), cv.w, cv.h, prec)
    f.set_tables(cv.pigtab, cv.cmf)
    f.write_state(cv.planes)
    f.update_params(2e-4, 1)
    for _ in range(4):
        f.encode_frame(1)
    return cv, f


def raw_state(f):
    """read_state in the reference layout (f16 pigments), as the 8 byte strings."""
    s = f.read_state(pig_format=capi.CF_PIG_F16)
    pig16 = np.asarray(s["strata_pig"], np.float32).astype(np.float16)
    return [np.ascontiguousarray(s["h"], np.float32).tobytes(), np.ascontiguousarray(s["m"], np.float32).tobytes(),
            np.ascontiguousarray(s["rheo"], np.float32).tobytes(), np.ascontiguousarray(s["strata_h"], np.float32).tobytes(),
            pig16.tobytes(), np.ascontiguousarray(s["strata_cure"], np.float32).tobytes(),
            np.asarray(s["sub_refl"], np.float32).astype(np.float16).tobytes(),
            np.ascontiguousarray(s["lay"], np.uint32).tobytes()]


@pytest.mark.parametrize("prec", [capi.CF_PREC_REFERENCE, capi.CF_PREC_FP32])
def test_save_parses_and_loads_back(built, prec):
    from canvaz_film.film import Film
    cv, f = stepped_film(prec)
    data = f.save_snapshot(h_max=1.5e-3, s_max=2.0, total_deposited=3.25e-6)
    hdr, parts = lz4_ref.parse_painting(data)
    assert (hdr["version"], hdr["w"], hdr["h"]) == (1, cv.w, cv.h)
    assert abs(hdr["h_max"] - 1.5e-3) < 1e-9 and hdr["total_deposited"] == 3.25e-6
    want = raw_state(f)
    assert [len(p) for p in parts] == [len(p) for p in want]
    for k, (a, b) in enumerate(zip(parts, want)):
        assert a == b, "part %d" % k
    # two films loaded from the file hold that state and step alike
    g1 = Film(po.make_settings(cv.settings), cv.w, cv.h, prec)
    g2 = Film(po.make_settings(cv.settings), cv.w, cv.h, prec)
    for g in (g1, g2):
        g.set_tables(cv.pigtab, cv.cmf)
        info = g.load_snapshot(data)
        assert info["w"] == cv.w and abs(info["s_max"] - 2.0) < 1e-9
        assert raw_state(g) == want
        g.update_params(2e-4, 1)
        for _ in range(3):
            g.encode_frame(1)
    assert raw_state(g1) == raw_state(g2)


def test_load_rejects_other_files(built):
    cv, f = stepped_film(capi.CF_PREC_REFERENCE)
    data = f.save_snapshot()
    from canvaz_film.film import Film
    from canvaz_film.capi import FilmError
    other = Film(po.make_settings(cv.settings), cv.w + 16, cv.h, capi.CF_PREC_REFERENCE)
    for bad in (b"NOPE" + data[4:], data[:40], data[:-10]):
        with pytest.raises(FilmError):
            f.load_snapshot(bad)
    with pytest.raises(FilmError):
        other.load_snapshot(data)


def test_load_rejects_sizes_the_file_cannot_back(built):
    """A damaged or hostile file that claims 2^32 - 1 chunks, or a chunk of
    more than 32 MiB raw, is refused with an error status, before the library
    allocates anything for those sizes."""
    import struct
    from canvaz_film.capi import FilmError
    cv, f = stepped_film(capi.CF_PREC_REFERENCE)
    data = f.save_snapshot()
    head = data[:44]
    many = head + struct.pack("<IQI", 8, 4 * cv.w * cv.h, 0xFFFFFFFF) + b"\0" * 64
    raw = head + struct.pack("<IQIQ", 8, 4 * cv.w * cv.h, 1, 8) + struct.pack("<I", 0xFFFFFFF0) + b"\0" * 4
    for bad in (many, raw):
        with pytest.raises(FilmError):
            f.load_snapshot(bad)
    f.load_snapshot(data)  # the film is still usable


def test_hand_written_painting_file_loads_and_saves(built):
    """The byte vector written from the format (tests/golden/psim_vector.py)
    loads into a 2 x 1 film as exactly its planes and header; the film saved
    again parses (independent parser) to the same header and planes."""
    import importlib.util
    from pathlib import Path
    import lz4_ref
    from canvaz_film.film import Film
    spec = importlib.util.spec_from_file_location("psim_vector", Path(__file__).parent / "golden" / "psim_vector.py")
    v = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(v)
    st = capi.Settings.default(width_m=2e-3, height_m=1e-3)
    f = Film(st, v.W, v.H, capi.CF_PREC_REFERENCE)
    cv = synth.blob_canvas(16, 16, 1, n_blobs=1, tables="reference")
    f.set_tables(cv.pigtab, cv.cmf)
    info = f.load_snapshot(v.FILE)
    assert (info["w"], info["h"]) == (v.W, v.H)
    for k, want in v.HEADER.items():
        assert np.float32(info[k]) == np.float32(want), k
    got = f.read_state(pig_format=capi.CF_PIG_F16)
    want = v.planes()
    for k in v.ORDER:  # read_state widens f16 slots and bands to f32, exactly
        np.testing.assert_array_equal(np.asarray(got[k]).reshape(-1),
                                      np.asarray(want[k]).astype(np.asarray(got[k]).dtype).reshape(-1), err_msg=k)
    data = f.save_snapshot(**{k: v.HEADER[k] for k in ("tilt_deg", "tilt_dir_deg", "cure_rate", "h_max", "s_max",
                                                       "total_deposited")})
    hdr, parts = lz4_ref.parse_painting(data)
    assert data[:44] == v.FILE[:44]
    assert parts == v.parts()
