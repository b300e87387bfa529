"""Extract the reference's own solver outputs from its README plan images.

The reference publishes four transport plans that its own solvers computed
on the README example (n = 100, m = 80), rendered by
figs/generate_readme_images.py of the reference (lines 21-62):

    plan_erot_bcd_reg0_1.png    sinkhorn_bcd(M, a, b, reg=0.1,  tol=1e-6, max_iter=1000)
    plan_erot_ssns_reg0_01.png  sinkhorn_ssns(M, a, b, reg=0.01, tol=1e-6, max_iter=1000)
    plan_qrot_pdip_reg0_1.png   qrot_pdip(M, a, b, reg=0.1,  tol=1e-8, inner_solver="cg")
    plan_qrot_pdip_reg0_01.png  qrot_pdip(M, a, b, reg=0.01, tol=1e-8, inner_solver="fp")

Each image is `imshow(T, cmap="viridis", interpolation="nearest")` of the
plan, so every plan entry is a uniform block of about 9 x 9 pixels whose
colour is the viridis entry floor(256 (T - min T) / (max T - min T)),
clipped to 255, truncated to 8 bits per channel. This script decodes the PNG
files (8-bit RGBA, no interlacing; a small zlib decoder, no imaging library),
finds the image area, reads the colour at the centre of every block, checks
that the block around it is uniform, and stores per image

    labels  (100, 80) uint8  colour class of each plan entry
    rgb     (K, 3)    uint8  the colour of each class

in reference_plan_images.npz beside this file, together with the solver call
that made the image. It needs the reference's figs/ directory and runs only
where the reference is checked out:

    python tests/golden/reference_images/make_reference_images.py [REFERENCE_DIR]
"""
import json
import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = "/root/reference"

# image file -> the call that produced it (figs/generate_readme_images.py:47-51)
IMAGES = {
    "plan_erot_bcd_reg0_1": ("sinkhorn_bcd", 0.1, 1e-6, 1000, {}),
    "plan_erot_ssns_reg0_01": ("sinkhorn_ssns", 0.01, 1e-6, 1000, {}),
    "plan_qrot_pdip_reg0_1": ("qrot_pdip", 0.1, 1e-8, 1000, {"inner_solver": "cg"}),
    "plan_qrot_pdip_reg0_01": ("qrot_pdip", 0.01, 1e-8, 1000, {"inner_solver": "fp"}),
}
N, M = 100, 80


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def read_png_rgba(path):
    """Decodes an 8-bit RGBA, non-interlaced PNG into an (h, w, 4) uint8 array."""
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        (ln,) = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + ln]
        pos += 12 + ln
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat.append(body)
    w, h, depth, ctype, _, _, interlace = hdr
    if (depth, ctype, interlace) != (8, 6, 0):
        raise ValueError(f"{path}: expected 8-bit RGBA without interlacing")
    raw = zlib.decompress(b"".join(idat))
    bpp, stride = 4, w * 4
    out = np.zeros((h, stride), np.int64)
    prev = np.zeros(stride, np.int64)
    for y in range(h):
        base = y * (stride + 1)
        ftype = raw[base]
        line = np.frombuffer(raw[base + 1:base + 1 + stride], np.uint8).astype(np.int64)
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(stride, np.int64)
            for x in range(stride):
                a = int(cur[x - bpp]) if x >= bpp else 0
                b = int(prev[x])
                c = int(prev[x - bpp]) if x >= bpp else 0
                pred = a if ftype == 1 else (a + b) // 2 if ftype == 3 else _paeth(a, b, c)
                cur[x] = (int(line[x]) + pred) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 4).astype(np.uint8)


def plan_cells(path, n=N, m=M):
    """Colour at the centre of each plan entry's block and the image area."""
    rgb = read_png_rgba(path)[..., :3].astype(np.int64)
    # the image area is the only large region of saturated colour (title,
    # ticks and frame are grey)
    sat = (rgb.max(-1) - rgb.min(-1)) > 10
    rows = np.where(sat.sum(1) > 100)[0]
    cols = np.where(sat.sum(0) > 100)[0]
    top, bottom, left, right = rows.min(), rows.max() + 1, cols.min(), cols.max() + 1
    bh, bw = (bottom - top) / n, (right - left) / m
    if not (8 <= bh <= 11 and 8 <= bw <= 11):
        raise ValueError(f"{path}: unexpected block size {bh} x {bw}")
    cells = np.zeros((n, m, 3), np.uint8)
    for i in range(n):
        y = int(top + (i + 0.5) * bh)
        for j in range(m):
            x = int(left + (j + 0.5) * bw)
            blk = rgb[y - 2:y + 3, x - 2:x + 3].reshape(-1, 3)
            if not (blk == blk[0]).all():
                raise ValueError(f"{path}: block ({i}, {j}) is not uniform")
            cells[i, j] = rgb[y, x]
    return cells, (int(top), int(bottom), int(left), int(right))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF
    out = {}
    for name, (solver, reg, tol, max_iter, kw) in IMAGES.items():
        cells, box = plan_cells(os.path.join(ref, "figs", name + ".png"))
        rgb, labels = np.unique(cells.reshape(-1, 3), axis=0, return_inverse=True)
        out[name + "/labels"] = labels.reshape(N, M).astype(np.uint8)
        out[name + "/rgb"] = rgb.astype(np.uint8)
        out[name + "/call"] = np.array(json.dumps(
            {"solver": solver, "reg": reg, "tol": tol, "max_iter": max_iter, "kwargs": kw,
             "n": N, "m": M, "image_box": box}))
        print(f"{name}: {len(rgb)} colours, image area rows {box[0]}-{box[1]}, "
              f"columns {box[2]}-{box[3]}")
    np.savez_compressed(os.path.join(HERE, "reference_plan_images.npz"), **out)


if __name__ == "__main__":
    main()
