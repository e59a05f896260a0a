"""Crop of the reference's own UHD plate-with-hole fixture, with its analytic truth.

The reference gates its full pyramid on the native UHD pair
assets/uhd_plate_hole/{reference,frame_095}.png (test_plate_hole.py:69-99,
UHDPlateRegressionTests): far-field population (radius >= 288 px), at least
90 % accepted, displacement RMSE below 0.05 px against the Kirsch solution at
250 MPa, and with roi_policy="partial" the 24 partial windows all accepted.
This script keeps a 768 x 768 window around the hole (origin a multiple of
the 16-px grid, so the subset lattice is the full image's), the hole mask of
that window and the truth at its subset centres, evaluated with the
reference's own tests/plate_hole_reference.py.  Run from the repository root
where the reference checkout is available:

    python tests/golden/make_plate_fixture.py /root/reference

PNG decoding is restated here (8-bit greyscale, non-interlaced: zlib inflate
plus the five scanline filters of the PNG specification) because Pillow is
not installed.  Output: tests/golden/plate_hole_crop.npz.
"""

from __future__ import annotations

import importlib.util
import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
X0, Y0, SIDE = 1536, 704, 768
SUBSET = 16
LOAD_MPA = 250.0


def read_png_gray8(path: Path) -> np.ndarray:
    data = path.read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path} is not a PNG file")
    pos, idat, header = 8, [], None
    while pos < len(data):
        length, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + length]
        if zlib.crc32(kind + body) & 0xFFFFFFFF != struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])[0]:
            raise ValueError(f"{path}: CRC mismatch in chunk {kind!r}")
        if kind == b"IHDR":
            header = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + length
    width, height, depth, colour, _, _, interlace = header
    if depth != 8 or colour != 0 or interlace != 0:
        raise ValueError(f"{path}: only 8-bit greyscale non-interlaced PNGs are handled")
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(height, width + 1)
    out = np.zeros((height, width), np.uint8)
    prev = np.zeros(width, np.int32)
    for r in range(height):
        kind, line = raw[r, 0], raw[r, 1:].astype(np.int32)
        if kind == 0:
            cur = line
        elif kind == 2:  # Up
            cur = (line + prev) & 255
        elif kind in (1, 3, 4):  # Sub, Average, Paeth: sequential in x
            cur = np.empty(width, np.int32)
            left = 0
            upleft = 0
            for x in range(width):
                up = int(prev[x])
                if kind == 1:
                    pred = left
                elif kind == 3:
                    pred = (left + up) >> 1
                else:
                    p = left + up - upleft
                    pa, pb, pc = abs(p - left), abs(p - up), abs(p - upleft)
                    pred = left if (pa <= pb and pa <= pc) else (up if pb <= pc else upleft)
                v = (int(line[x]) + pred) & 255
                cur[x] = v
                left, upleft = v, up
        else:
            raise ValueError(f"{path}: unknown filter {kind}")
        out[r] = cur
        prev = cur
    return out


def main(reference_root: str) -> None:
    root = Path(reference_root) / "DIC" / "LucasKanadeICGN"
    assets = root / "assets" / "uhd_plate_hole"
    spec = importlib.util.spec_from_file_location("plate_hole_reference",
                                                  root / "python" / "tests" / "plate_hole_reference.py")
    phr = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(phr)
    reference = read_png_gray8(assets / "reference.png")
    target = read_png_gray8(assets / "frame_095.png")
    assert reference.shape == (phr.HEIGHT, phr.WIDTH) and target.shape == reference.shape
    crop = np.s_[Y0:Y0 + SIDE, X0:X0 + SIDE]
    mask = phr.hole_mask()[crop]
    gy, gx = np.indices(((SIDE - SUBSET) // SUBSET + 1, (SIDE - SUBSET) // SUBSET + 1))
    cx, cy = gx * SUBSET + (SUBSET - 1) / 2, gy * SUBSET + (SUBSET - 1) / 2
    truth = phr.displacement(cx + X0, cy + Y0, LOAD_MPA)
    np.savez_compressed(
        HERE / "plate_hole_crop.npz",
        reference=np.ascontiguousarray(reference[crop]), target=np.ascontiguousarray(target[crop]),
        mask=np.ascontiguousarray(mask), origin=np.array([X0, Y0]), centre=np.array([phr.CX, phr.CY]),
        radius=np.array(phr.RADIUS), truth=truth, load_mpa=np.array(LOAD_MPA),
        full_partial_count=np.array(24))
    print("wrote", HERE / "plate_hole_crop.npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
