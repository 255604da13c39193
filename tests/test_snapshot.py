"""The painting-file chunk coder (cf_lz4_*) on CPU: round trips, decoding by
an independent LZ4 block decoder, a hand-built block, malformed input."""
import ctypes as C
import struct

import numpy as np
import pytest

import lz4_ref
from canvaz_film import capi


@pytest.fixture(scope="module")
def lib():
    if not capi.LIB_PATH.exists():
        import __graft_entry__ as g
        g.build()
    L = capi.load_library()
    for name in ("cf_lz4_compress", "cf_lz4_decompress"):
        fn = getattr(L, name)
        fn.argtypes = [C.c_char_p, C.c_uint64, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
        fn.restype = C.c_int32
    return L


def compress(L, data):
    cap = len(data) + len(data) // 255 + 64
    out = C.create_string_buffer(cap)
    n = C.c_uint64()
    assert L.cf_lz4_compress(data, len(data), out, cap, C.byref(n)) == capi.CF_OK
    return out.raw[: n.value]


def decompress(L, chunk):
    n = C.c_uint64()
    assert L.cf_lz4_decompress(chunk, len(chunk), None, 0, C.byref(n)) == capi.CF_OK
    out = C.create_string_buffer(max(n.value, 1))
    st = L.cf_lz4_decompress(chunk, len(chunk), out, n.value, C.byref(n))
    return st, out.raw[: n.value]


def inputs():
    rng = np.random.default_rng(7)
    yield b""
    for k in (1, 4, 5, 12, 13, 17, 64):
        yield bytes(rng.integers(0, 256, k, dtype=np.uint8))
    yield b"\x00" * 100000
    yield b"abcd" * 5000
    yield bytes(rng.integers(0, 256, 70000, dtype=np.uint8))
    # float planes like the state: smooth field with repeats and zeros
    h = np.zeros(300000, np.float32)
    h[1000:50000] = np.linspace(0, 1e-3, 49000, dtype=np.float32)
    yield h.tobytes()
    yield (np.arange(200000) % 300).astype(np.uint16).tobytes()


def test_round_trip_and_independent_decoder(lib):
    for data in inputs():
        chunk = compress(lib, data)
        assert struct.unpack_from("<I", chunk)[0] == len(data)
        assert lz4_ref.decompress_size_prepended(chunk) == data
        st, back = decompress(lib, chunk)
        assert st == capi.CF_OK and back == data
    # repetitive data compresses
    assert len(compress(lib, b"\x00" * 100000)) < 1000


def test_decodes_blocks_it_did_not_write(lib):
    # literal run + a match (offset 4, length 8) + the last 5 literals
    block = bytes([0x44]) + b"abcd" + bytes([4, 0]) + bytes([0x50]) + b"xyz12"
    chunk = struct.pack("<I", 17) + block
    assert lz4_ref.decompress_size_prepended(chunk) == b"abcdabcdabcdxyz12"
    st, back = decompress(lib, chunk)
    assert st == capi.CF_OK and back == b"abcdabcdabcdxyz12"
    data = bytes(range(256)) * 3
    st, back = decompress(lib, lz4_ref.literal_only_chunk(data))
    assert st == capi.CF_OK and back == data


def test_rejects_malformed_blocks(lib):
    bad = [
        struct.pack("<I", 8) + bytes([0x40]) + b"abcd" + bytes([0, 0]) + bytes([0x00]),   # offset 0
        struct.pack("<I", 8) + bytes([0x40]) + b"abcd" + bytes([9, 0]) + bytes([0x00]),   # offset past output
        struct.pack("<I", 8) + bytes([0x80]) + b"abc",                                     # literals past the end
        struct.pack("<I", 99) + bytes([0x40]) + b"abcd",                                   # wrong size
    ]
    for chunk in bad:
        st, _ = decompress(lib, chunk)
        assert st == capi.CF_ERR_INVALID_ARG


def _vector():
    import importlib.util
    from pathlib import Path
    spec = importlib.util.spec_from_file_location("psim_vector", Path(__file__).parent / "golden" / "psim_vector.py")
    v = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(v)
    return v


def test_hand_written_painting_file_parses():
    """The byte vector written from the format (tests/golden/psim_vector.py)
    parses with the independent parser into the header and the 8 planes."""
    v = _vector()
    hdr, parts = lz4_ref.parse_painting(v.FILE)
    assert hdr["version"] == 1 and (hdr["w"], hdr["h"]) == (v.W, v.H)
    for k, want in v.HEADER.items():
        assert np.float64(hdr[k]) == np.float64(np.float32(want)) or hdr[k] == want, k
    assert parts == v.parts()


def test_hand_written_blocks_decode_in_the_library(lib):
    """Each hand-written chunk (literal runs, zero runs at offset 1, an f16
    pattern at offset 2, length bytes in both nibbles) decodes in the
    library's own LZ4 decoder to its plane."""
    v = _vector()
    for (off, clen), want in zip(v.chunks(), v.parts()):
        st, back = decompress(lib, v.FILE[off:off + clen])
        assert st == capi.CF_OK and back == want
