"""Windows of the reference's own native UHD fixtures, with their truth.

Plate with hole.
The reference gates its full pyramid on the native UHD pair
assets/uhd_plate_hole/{reference,frame_095}.png (test_plate_hole.py:69-99,
UHDPlateRegressionTests): far-field population (radius >= 288 px), at least
90 % accepted, displacement RMSE below 0.05 px against the Kirsch solution at
250 MPa, and with roi_policy="partial" the 24 partial windows all accepted.
This script keeps a 768 x 768 window around the hole (origin a multiple of
the 16-px grid, so the subset lattice is the full image's), the hole mask of
that window and the truth at its subset centres, evaluated with the
reference's own tests/plate_hole_reference.py.

Tensile.  The reference's UHD tensile regressions (test_uhd_fixtures.py:
UHDRegistrationRegressionTests, 316-406) register assets/uhd_tensile/
frame_040.png against reference.png with S16/s16 (uniform stretch about the
frame centre from machine_truth.csv, limits from manifest.json's
regression_limits) and recover the identity on every archived image.  This
script keeps a 768 x 768 window of reference.png and frame_040.png (origin
on the 16-px grid, away from the centre so the stretch displaces it by 1 to
1.9 px), the stretches of frame 40 and the limits, and the same window of
the reference under the large fractional translations of the 4-level
pyramid and Fourier-initialisation regressions (test_uhd_fixtures.py:86-128),
rendered from the full frame by the reference's own fractional_shift.

Run from the repository root where the reference checkout is available:

    python tests/golden/make_uhd_fixtures.py <path of the live-dic checkout>

PNG decoding is restated here (8-bit greyscale, non-interlaced: zlib inflate
plus the five scanline filters of the PNG specification) because Pillow is
not installed.  Outputs: tests/golden/plate_hole_crop.npz, tests/golden/tensile_crop.npz.
"""

from __future__ import annotations

import csv
import importlib.util
import json
import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
X0, Y0, SIDE = 1536, 704, 768
SUBSET = 16
LOAD_MPA = 250.0
TX0, TY0 = 2816, 1280
SHIFT_PYRAMID, SHIFT_FOURIER = (16.35, -8.2), (128.35, -64.2)


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


def tensile(root: Path) -> None:
    assets = root / "assets" / "uhd_tensile"
    manifest = json.loads((assets / "manifest.json").read_text())
    with (assets / "machine_truth.csv").open(newline="") as stream:
        row = {int(r["frame"]): r for r in csv.DictReader(stream)}[40]
    reference = read_png_gray8(assets / "reference.png")
    target = read_png_gray8(assets / "frame_040.png")
    assert reference.shape == (manifest["height"], manifest["width"]) == target.shape
    crop = np.s_[TY0:TY0 + SIDE, TX0:TX0 + SIDE]
    limits = manifest["regression_limits"]
    # Large fractional rigid motion rendered from the full reference by the
    # reference's own generator (uhd_partial_cases.fractional_shift), then cut.
    sys.path.insert(0, str(HERE))
    from make_golden import _import_reference

    _import_reference(root.parents[1])
    import uhd_partial_cases

    shifted = {name: uhd_partial_cases.fractional_shift(reference, motion)[crop]
               for name, motion in (("shift_pyramid", SHIFT_PYRAMID), ("shift_fourier", SHIFT_FOURIER))}
    np.savez_compressed(
        HERE / "tensile_crop.npz",
        reference=np.ascontiguousarray(reference[crop]), target=np.ascontiguousarray(target[crop]),
        shift_pyramid=np.ascontiguousarray(shifted["shift_pyramid"]), motion_pyramid=np.array(SHIFT_PYRAMID),
        shift_fourier=np.ascontiguousarray(shifted["shift_fourier"]), motion_fourier=np.array(SHIFT_FOURIER),
        origin=np.array([TX0, TY0]), centre=np.array([1920.0, 1080.0]),
        stretch=np.array([float(row["stretch_x"]), float(row["stretch_y"])]),
        limit_names=np.array(sorted(limits)), limit_values=np.array([float(limits[k]) for k in sorted(limits)]))
    print("wrote", HERE / "tensile_crop.npz")


def main(reference_root: str) -> None:
    root = Path(reference_root) / "DIC" / "LucasKanadeICGN"
    tensile(root)
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
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {sys.argv[0]} <path of the live-dic checkout>")
    main(sys.argv[1])
