"""Consistency of a transport plan with the reference's rendered plan images.

The reference renders the plans of four of its own solves with matplotlib's
`imshow(T, cmap="viridis", interpolation="nearest")` (figs/
generate_readme_images.py:35-39 of the reference). matplotlib normalises the
plan linearly onto [0, 1] by its minimum and maximum, picks the colormap
entry floor(256 v), 255 for v = 1 (Colormap.__call__), and truncates the
entry to 8 bits per channel. tests/golden/reference_images/ stores the colour
of every plan entry read back from those images.

The check below needs no copy of the colormap. It uses three properties of
viridis and of the rendering:
  - viridis's green channel rises monotonically from its first entry to its
    last, so colour classes sorted by plan value must have nondecreasing
    green;
  - two different colours are two different colormap entries, so all entries
    of one colour class lie in bins strictly below those of the next class;
  - after truncation to 8 bits two adjacent colormap entries can share a
    colour, so one class may cover two adjacent bins, never more.
With tol = 0 every plan entry must fall in the bin its colour allows; a tol
(in bins, 1 bin = 1/256 of the plan's range) excuses entries that lie within
tol of a bin edge, for plans that differ from the reference's solve by
rounding or by the stopping point.
"""
import json
import os

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_images",
                       "reference_plan_images.npz")
IMAGES = ("plan_erot_bcd_reg0_1", "plan_erot_ssns_reg0_01", "plan_qrot_pdip_reg0_1",
          "plan_qrot_pdip_reg0_01")


def load(name):
    """(labels, rgb, call) of one image: the colour class of every plan entry,
    the colour of each class, and the reference's solver call that made it."""
    g = np.load(FIXTURE)
    return g[name + "/labels"], g[name + "/rgb"], json.loads(str(g[name + "/call"]))


def _bins(x, tol):
    """Lowest and highest colormap bin of each value moved by up to tol bins."""
    lo = np.clip(np.floor(x - tol), 0, 255)
    hi = np.clip(np.floor(x + tol), 0, 255)
    return lo, hi


def violations(T, labels, rgb, tol=0.0):
    """Number of broken constraints between the plan T and the image."""
    T = np.asarray(T, dtype=np.float64)
    if T.shape != labels.shape:
        raise ValueError(f"plan shape {T.shape} against image {labels.shape}")
    span = T.max() - T.min()
    x = 256.0 * (T - T.min()) / span if span > 0 else np.zeros_like(T)
    lo, hi = _bins(x, tol)
    k = len(rgb)
    order = sorted(range(k), key=lambda c: float(np.median(x[labels == c])))
    bad = 0
    green = rgb[order, 1].astype(np.int64)
    bad += int(np.sum(np.diff(green) < 0))
    floor_top, ceil_bottom = [], []
    for c in order:
        sel = labels == c
        # the class's highest entry sits at least at floor_top, its lowest at
        # most at ceil_bottom; one colour covers at most two adjacent bins
        ft, cb = lo[sel].max(), hi[sel].min()
        bad += int(ft - cb > 1)
        floor_top.append(ft)
        ceil_bottom.append(cb)
    for c in range(k - 1):
        bad += int(not floor_top[c] < ceil_bottom[c + 1])
    return bad


def needed_tol(T, labels, rgb):
    """The smallest tolerance (in bins) from a fixed ladder at which T agrees
    with the image, or inf."""
    for tol in (0.0, 1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 3e-2, 1e-1, 3e-1):
        if violations(T, labels, rgb, tol) == 0:
            return tol
    return float("inf")
