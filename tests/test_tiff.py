"""The TIFF volume reader (CPU only): round trips through the writer, hand-built big-endian and
PackBits files, rejection of unsupported files, and the reference's own example volume
(docs/paper/TF-500x500x500-1x2x6-v3.tiff.zip) when its source tree is present."""
import os
import struct
import zipfile

import numpy as np
import pytest

from taufactor_gb300.tiff import read_tiff, unpack_bits, write_tiff


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.int16, np.float32])
def test_round_trip(tmp_path, dtype):
    rng = np.random.default_rng(3)
    vol = (rng.random((5, 7, 9)) * 200).astype(dtype)
    p = tmp_path / "v.tif"
    write_tiff(p, vol)
    out = read_tiff(p)
    assert out.dtype == vol.dtype and out.shape == vol.shape
    np.testing.assert_array_equal(out, vol)


def test_single_page_and_bytes(tmp_path):
    img = np.arange(12, dtype=np.uint8).reshape(3, 4)
    p = tmp_path / "one.tif"
    write_tiff(p, img)
    np.testing.assert_array_equal(read_tiff(p), img[None])
    np.testing.assert_array_equal(read_tiff(p.read_bytes()), img[None])


def test_zip_member(tmp_path):
    vol = (np.arange(2 * 3 * 4) % 2 * 255).astype(np.uint8).reshape(2, 3, 4)
    write_tiff(tmp_path / "v.tif", vol)
    z = tmp_path / "v.tiff.zip"
    with zipfile.ZipFile(z, "w", compression=zipfile.ZIP_DEFLATED) as f:
        f.writestr("__MACOSX/._v.tif", b"resource fork")
        f.write(tmp_path / "v.tif", "v.tif")
    np.testing.assert_array_equal(read_tiff(z), vol)


def _strip_tiff(e, pages, strip_rows, packbits=False):
    """Hand-built multi-page 16-bit TIFF in byte order `e`, several strips per page, with
    out-of-line strip tables (the layout of the reference's example volume)."""
    h, w = pages[0].shape
    body = bytearray(b"II" if e == "<" else b"MM")
    body += struct.pack(e + "HI", 42, 0)
    ifds = []
    for img in pages:
        offs, cnts = [], []
        for r0 in range(0, h, strip_rows):
            raw = img[r0:r0 + strip_rows].astype(e + "u2").tobytes()
            if packbits:  # literal runs of at most 128 bytes
                enc = bytearray()
                for i in range(0, len(raw), 128):
                    part = raw[i:i + 128]
                    enc += bytes([len(part) - 1]) + part
                raw = bytes(enc)
            offs.append(len(body))
            cnts.append(len(raw))
            body += raw
        if len(body) % 2:
            body += b"\0"
        n = len(offs)
        off_tab = len(body)
        body += struct.pack(e + "I" * n, *offs)
        cnt_tab = len(body)
        body += struct.pack(e + "I" * n, *cnts)
        ifds.append(len(body))
        ent = [(256, 3, 1, struct.pack(e + "HH", w, 0)), (257, 3, 1, struct.pack(e + "HH", h, 0)),
               (258, 3, 1, struct.pack(e + "HH", 16, 0)), (259, 3, 1, struct.pack(e + "HH", 32773 if packbits else 1, 0)),
               (273, 4, n, struct.pack(e + "I", off_tab)), (278, 3, 1, struct.pack(e + "HH", strip_rows, 0)),
               (279, 4, n, struct.pack(e + "I", cnt_tab))]
        body += struct.pack(e + "H", len(ent))
        for t, typ, c, val in ent:
            body += struct.pack(e + "HHI", t, typ, c) + val
        body += struct.pack(e + "I", 0)
    struct.pack_into(e + "I", body, 4, ifds[0])
    for a, b in zip(ifds, ifds[1:]):
        n = struct.unpack_from(e + "H", body, a)[0]
        struct.pack_into(e + "I", body, a + 2 + 12 * n, b)
    return bytes(body)


@pytest.mark.parametrize("e", ["<", ">"])
@pytest.mark.parametrize("packbits", [False, True])
def test_strips_byte_order_packbits(e, packbits):
    rng = np.random.default_rng(5)
    pages = [rng.integers(0, 65535, (11, 13)).astype(np.uint16) for _ in range(3)]
    out = read_tiff(_strip_tiff(e, pages, strip_rows=4, packbits=packbits))
    assert out.dtype == np.uint16
    np.testing.assert_array_equal(out, np.stack(pages))


def test_unpack_bits_spec_example():
    # the worked example of the PackBits scheme (TIFF 6.0, section 9)
    packed = bytes.fromhex("FEAA0280002AFDAA0380002A22F7AA")
    expect = bytes.fromhex("AAAAAA80002AAAAAAAAA80002A22AAAAAAAAAAAAAAAAAAAA")
    assert unpack_bits(packed, len(expect)) == expect


def test_rejects():
    with pytest.raises(ValueError):
        read_tiff(b"PK\x03\x04 not a tiff")
    with pytest.raises(ValueError):
        read_tiff(b"II" + struct.pack("<HI", 43, 8))  # BigTIFF
    img = np.zeros((2, 2), np.uint8)
    good = bytearray(_strip_tiff("<", [img.astype(np.uint16)], 2))
    # point the first IFD at itself through its next-IFD field: a cycle
    first = struct.unpack_from("<I", good, 4)[0]
    n = struct.unpack_from("<H", good, first)[0]
    struct.pack_into("<I", good, first + 2 + 12 * n, first)
    with pytest.raises(ValueError):
        read_tiff(bytes(good))


def test_reference_example_volume():
    from oracle.ref_shim import reference_root

    root = reference_root()
    path = None if root is None else os.path.join(root, "docs", "paper", "TF-500x500x500-1x2x6-v3.tiff.zip")
    if path is None or not os.path.exists(path):
        pytest.skip("reference source tree absent")
    vol = read_tiff(path)
    assert vol.shape == (500, 500, 500) and vol.dtype == np.uint8
    labels, counts = np.unique(vol, return_counts=True)
    assert labels.tolist() == [0, 255]
    # 30 % of the voxels are the 255 phase
    assert counts.tolist() == [87_500_000, 37_500_000]
