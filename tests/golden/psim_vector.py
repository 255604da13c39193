"""A painting file written byte by byte: the pin of the format.

A 2 x 1 canvas saved as the reference saves it (src/session.rs:248-275 for
the header, pack() at src/session.rs:59-72 for the parts): the 44-byte
header, the part count, then for each of the 8 read_state planes its length
(u64), its chunk count (u32) and each chunk as a u64 length followed by a
size-prepended LZ4 block (lz4_flex::compress_prepend_size: the raw size as
u32, then the block).  All integers and floats are little-endian.

The LZ4 blocks are written by hand from the LZ4 block format: a block is a
series of sequences; a sequence is a token (high nibble: literal count, low
nibble: match length - 4; 15 in a nibble means that more length bytes follow,
each added, until one below 255), the literals, then a 2-byte offset back
into the output and the match bytes, copied one at a time, so an offset
shorter than the match repeats a pattern.  The last sequence has literals
only, the last 5 bytes of a block are literals, and the last match starts at
least 12 bytes before the end of the block.  The blocks below use literal-only
runs (8 and 16 bytes, the 16 with a length byte), runs of zeros copied at
offset 1 with extra length bytes, and a 2-byte f16 pattern copied at
offset 2.
"""
import struct

import numpy as np

W, H = 2, 1
HEADER = {"tilt_deg": 60.0, "tilt_dir_deg": 90.0, "cure_rate": 0.5, "h_max": np.float32(1e-3), "s_max": 1.0,
          "total_deposited": 3.0}


def _hex(s):
    return bytes.fromhex(s.replace("\n", " "))


FILE = _hex("""
50 53 49 4d  01 00 00 00  02 00 00 00  01 00 00 00
00 00 70 42  00 00 b4 42  00 00 00 3f  6f 12 83 3a  00 00 80 3f
00 00 00 00 00 00 08 40
08 00 00 00
08 00 00 00 00 00 00 00  01 00 00 00  0d 00 00 00 00 00 00 00
  08 00 00 00  80  6f 12 83 3a 00 00 00 00
08 00 00 00 00 00 00 00  01 00 00 00  0d 00 00 00 00 00 00 00
  08 00 00 00  80  00 00 00 00 00 00 00 00
10 00 00 00 00 00 00 00  01 00 00 00  16 00 00 00 00 00 00 00
  10 00 00 00  f0 01  00 00 80 3f 00 00 00 00 00 00 80 3f 00 00 00 00
20 00 00 00 00 00 00 00  01 00 00 00  13 00 00 00 00 00 00 00
  20 00 00 00  5f  6f 12 83 3a 00  01 00  03  50  00 00 00 00 00
00 01 00 00 00 00 00 00  01 00 00 00  11 00 00 00 00 00 00 00
  00 01 00 00  3f  00 3c 00  01 00  e5  50  00 00 00 00 00
20 00 00 00 00 00 00 00  01 00 00 00  0f 00 00 00 00 00 00 00
  20 00 00 00  1f  00  01 00  07  50  00 00 00 00 00
40 00 00 00 00 00 00 00  01 00 00 00  10 00 00 00 00 00 00 00
  40 00 00 00  2f  00 38  02 00  26  50  38 00 38 00 38
08 00 00 00 00 00 00 00  01 00 00 00  0d 00 00 00 00 00 00 00
  08 00 00 00  80  02 00 00 00 00 00 00 00
""")


def planes():
    """The state the file holds, in write_state's layout."""
    h = np.array([1e-3, 0.0], np.float32)
    m = np.zeros(2, np.float32)
    rheo = np.array([[1.0, 0.0], [1.0, 0.0]], np.float32)
    strata_h = np.zeros((2, 4), np.float32)
    strata_h[0, 0] = np.float32(1e-3)
    pig = np.zeros((2, 64), np.float16)
    pig[0, 0] = 1.0
    cure = np.zeros((2, 4), np.float32)
    sub = np.full((2, 16), 0.5, np.float16)
    lay = np.array([2, 0], np.uint32)
    return {"h": h, "m": m, "rheo": rheo, "strata_h": strata_h, "strata_pig": pig, "strata_cure": cure,
            "sub_refl": sub, "lay": lay}


ORDER = ["h", "m", "rheo", "strata_h", "strata_pig", "strata_cure", "sub_refl", "lay"]


def parts():
    p = planes()
    return [np.ascontiguousarray(p[k]).tobytes() for k in ORDER]


def chunks():
    """(offset, length) of each size-prepended chunk in FILE, in part order."""
    out, off = [], 44 + 4
    for _ in range(8):
        _, nch = struct.unpack_from("<QI", FILE, off)
        off += 12
        for _ in range(nch):
            (clen,) = struct.unpack_from("<Q", FILE, off)
            out.append((off + 8, clen))
            off += 8 + clen
    assert off == len(FILE)
    return out
