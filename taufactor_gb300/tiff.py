"""Multi-page TIFF volumes with the standard library and numpy (the on-disk format of the
reference's example volume, docs/paper/TF-500x500x500-1x2x6-v3.tiff.zip; the reference itself
reads such files through third-party packages in its notebooks).

Reads classic TIFF (little or big endian): one grayscale sample per pixel of 8, 16 or 32 bits
(unsigned, signed or IEEE float), strips or whole pages, uncompressed or PackBits; page p is slice
[p] of the returned array [pages, rows, columns]. A ``.zip`` path reads the first TIFF member of
the archive. ``write_tiff`` writes the uncompressed little-endian form.
"""
from __future__ import annotations

import io
import os
import struct
import zipfile

import numpy as np

_TYPE_FORMAT = {1: "B", 2: "c", 3: "H", 4: "I", 5: "II", 6: "b", 8: "h", 9: "i", 11: "f", 12: "d", 16: "Q"}
_TYPE_SIZE = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 6: 1, 7: 1, 8: 2, 9: 4, 10: 8, 11: 4, 12: 8, 16: 8}
_SAMPLE_KIND = {1: "u", 2: "i", 3: "f"}


def _tag_values(data: bytes, e: str, typ: int, cnt: int, field: bytes):
    size = _TYPE_SIZE.get(typ, 1) * cnt
    if size <= 4:
        raw = field[:size]
    else:
        o = struct.unpack(e + "I", field)[0]
        raw = bytes(data[o:o + size])
    if typ in (5, 10):  # rationals: pairs
        vals = struct.unpack(e + ("I" if typ == 5 else "i") * (2 * cnt), raw)
        return [vals[2 * i] / vals[2 * i + 1] if vals[2 * i + 1] else 0.0 for i in range(cnt)]
    fmt = _TYPE_FORMAT.get(typ)
    if fmt is None or typ in (2, 7):
        return raw
    return list(struct.unpack(e + fmt * cnt, raw))


def unpack_bits(buf: bytes, size: int) -> bytes:
    """PackBits decoding (TIFF 6.0, section 9) up to `size` bytes."""
    out = bytearray()
    i, n = 0, len(buf)
    while i < n and len(out) < size:
        h = buf[i]
        i += 1
        if h < 128:  # literal run of h + 1 bytes
            out += buf[i:i + h + 1]
            i += h + 1
        elif h > 128:  # repeat the next byte 257 - h times
            out += bytes([buf[i]]) * (257 - h)
            i += 1
    return bytes(out[:size])


def _read_bytes(source) -> bytes:
    if isinstance(source, (bytes, bytearray)):
        return bytes(source)
    path = os.fspath(source)
    if path.lower().endswith(".zip"):
        with zipfile.ZipFile(path) as z:
            names = [n for n in z.namelist()
                     if n.lower().endswith((".tif", ".tiff")) and not os.path.basename(n).startswith("._")]
            if not names:
                raise ValueError(f"{path}: no TIFF member")
            return z.read(names[0])
    with open(path, "rb") as f:
        return f.read()


def read_tiff(source) -> np.ndarray:
    """Volume [pages, rows, columns] from a multi-page grayscale TIFF (path, .zip path or bytes)."""
    data = memoryview(_read_bytes(source))
    if data[:2] == b"II":
        e = "<"
    elif data[:2] == b"MM":
        e = ">"
    else:
        raise ValueError("not a TIFF file")
    if struct.unpack(e + "H", data[2:4])[0] != 42:
        raise ValueError("only classic TIFF is supported (not BigTIFF)")
    off = struct.unpack(e + "I", data[4:8])[0]
    pages = []
    seen = set()
    while off:
        if off in seen or off + 2 > len(data):
            raise ValueError("corrupt IFD chain")
        seen.add(off)
        n = struct.unpack(e + "H", data[off:off + 2])[0]
        tags = {}
        for i in range(n):
            ent = data[off + 2 + 12 * i: off + 14 + 12 * i]
            t, typ, cnt = struct.unpack(e + "HHI", ent[:8])
            tags[t] = _tag_values(data, e, typ, cnt, ent[8:12])
        pages.append(_decode_page(data, e, tags))
        off = struct.unpack(e + "I", data[off + 2 + 12 * n: off + 6 + 12 * n])[0]
    if not pages:
        raise ValueError("no image in TIFF")
    if any(p.shape != pages[0].shape or p.dtype != pages[0].dtype for p in pages):
        raise ValueError("pages differ in shape or type")
    return np.stack(pages)


def _decode_page(data: bytes, e: str, tags: dict) -> np.ndarray:
    width, height = tags[256][0], tags[257][0]
    bits = tags.get(258, [1])[0]
    if tags.get(277, [1])[0] != 1:
        raise ValueError("only one sample per pixel is supported")
    comp = tags.get(259, [1])[0]
    if comp not in (1, 32773):
        raise ValueError(f"compression {comp} is not supported (uncompressed or PackBits only)")
    kind = _SAMPLE_KIND.get(tags.get(339, [1])[0], "u")
    if bits not in (8, 16, 32):
        raise ValueError(f"{bits}-bit samples are not supported")
    dtype = np.dtype(f"{e}{kind}{bits // 8}")
    offsets, counts = tags[273], tags[279]
    rows = tags.get(278, [height])[0]
    need = width * height * dtype.itemsize
    out = np.empty(need, np.uint8)
    pos = 0
    for k, (o, c) in enumerate(zip(offsets, counts)):
        chunk = data[o:o + c]
        if comp == 32773:
            nrows = min(rows, height - k * rows)
            chunk = unpack_bits(bytes(chunk), nrows * width * dtype.itemsize)
        take = min(len(chunk), need - pos)
        out[pos:pos + take] = np.frombuffer(chunk, np.uint8, count=take)
        pos += take
        if pos == need:
            break
    if pos < need:
        raise ValueError("truncated image data")
    return out.view(dtype).reshape(height, width).astype(dtype.newbyteorder("="))


def write_tiff(path, volume) -> None:
    """Uncompressed little-endian multi-page TIFF, one page per slice of volume [pages, rows, cols]
    (uint8/uint16/uint32/int*/float32)."""
    v = np.ascontiguousarray(volume)
    if v.ndim == 2:
        v = v[None]
    if v.ndim != 3:
        raise ValueError("volume must be 2-D or 3-D")
    if v.dtype.kind not in "uif" or v.dtype.itemsize not in (1, 2, 4):
        raise ValueError(f"unsupported dtype {v.dtype}")
    v = v.astype(v.dtype.newbyteorder("<"))
    fmt = {"u": 1, "i": 2, "f": 3}[v.dtype.kind]
    pages, height, width = v.shape
    buf = io.BytesIO()
    buf.write(b"II" + struct.pack("<HI", 42, 0))
    ifd_pos = []
    for p in range(pages):
        img_off = buf.tell()
        buf.write(v[p].tobytes())
        if buf.tell() % 2:
            buf.write(b"\0")
        ifd = buf.tell()
        ifd_pos.append(ifd)
        entries = [(256, 4, width), (257, 4, height), (258, 3, v.dtype.itemsize * 8), (259, 3, 1), (262, 3, 1),
                   (273, 4, img_off), (277, 3, 1), (278, 4, height), (279, 4, v[p].nbytes), (339, 3, fmt)]
        buf.write(struct.pack("<H", len(entries)))
        for t, typ, val in entries:
            buf.write(struct.pack("<HHI", t, typ, 1) + (struct.pack("<HH", val, 0) if typ == 3 else struct.pack("<I", val)))
        buf.write(struct.pack("<I", 0))
    raw = bytearray(buf.getvalue())
    struct.pack_into("<I", raw, 4, ifd_pos[0])
    for a, b in zip(ifd_pos, ifd_pos[1:]):
        n = struct.unpack_from("<H", raw, a)[0]
        struct.pack_into("<I", raw, a + 2 + 12 * n, b)
    with open(path, "wb") as f:
        f.write(bytes(raw))
