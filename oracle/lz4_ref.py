"""Independent restatement of the painting-file format (src/session.rs:6-99,
248-310) and of the LZ4 block format it stores its chunks in.

TEST INFRASTRUCTURE: the checker of the library's cf_snapshot_* / cf_lz4_*
(written from the published LZ4 block format, not from the library's code);
never used on the product path.
"""
import struct


def lz4_block_decode(src, out_len):
    """Decodes an LZ4 block to exactly out_len bytes (raises on malformed input)."""
    out = bytearray()
    ip, n = 0, len(src)
    while ip < n:
        token = src[ip]
        ip += 1
        lit = token >> 4
        if lit == 15:
            while True:
                b = src[ip]
                ip += 1
                lit += b
                if b != 255:
                    break
        if ip + lit > n:
            raise ValueError("literals past the end")
        out += src[ip:ip + lit]
        ip += lit
        if ip == n:
            break
        off = src[ip] | (src[ip + 1] << 8)
        ip += 2
        if off == 0 or off > len(out):
            raise ValueError("bad offset")
        ml = token & 15
        if ml == 15:
            while True:
                b = src[ip]
                ip += 1
                ml += b
                if b != 255:
                    break
        ml += 4
        for _ in range(ml):
            out.append(out[-off])
    if len(out) != out_len:
        raise ValueError("decoded %d bytes, expected %d" % (len(out), out_len))
    return bytes(out)


def decompress_size_prepended(chunk):
    (n,) = struct.unpack_from("<I", chunk, 0)
    return lz4_block_decode(chunk[4:], n)


def literal_only_chunk(data):
    """A valid size-prepended LZ4 chunk holding `data` as one literal run."""
    lit = len(data)
    token = bytes([min(lit, 15) << 4])
    ext = b""
    if lit >= 15:
        rest = lit - 15
        ext = b"\xff" * (rest // 255) + bytes([rest % 255])
    return struct.pack("<I", lit) + token + ext + bytes(data)


HEADER = struct.Struct("<4sIII5fd")  # 44 bytes


def parse_painting(data):
    """(header dict, [8 parts]) of a painting file."""
    magic, ver, w, h, tilt, tdir, cure, hmax, smax, dep = HEADER.unpack_from(data, 0)
    assert magic == b"PSIM"
    hdr = dict(version=ver, w=w, h=h, tilt_deg=tilt, tilt_dir_deg=tdir, cure_rate=cure, h_max=hmax, s_max=smax,
               total_deposited=dep)
    off = HEADER.size
    (count,) = struct.unpack_from("<I", data, off)
    off += 4
    parts = []
    for _ in range(count):
        length, nch = struct.unpack_from("<QI", data, off)
        off += 12
        buf = bytearray()
        for _ in range(nch):
            (clen,) = struct.unpack_from("<Q", data, off)
            off += 8
            buf += decompress_size_prepended(data[off:off + clen])
            off += clen
        assert len(buf) == length
        parts.append(bytes(buf))
    assert off == len(data)
    return hdr, parts
