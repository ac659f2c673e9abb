"""The tiled mixed explicit step's copy windows (csrc/explicit.cu: tile_win, stage_bytes),
restated and checked for every tile position of many array sizes: each bulk copy starts
on a 16-byte boundary, has a 16-byte multiple size, fits its shared-memory region, stays
inside its array rounded up to 16 bytes (the arena pads every array to 256), and covers
every element (and neighbour) the step reads from it."""
import os
import random
import re

import pytest

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "168861_gb300", "csrc", "explicit.cu")


def constants():
    src = open(SRC).read()
    te = int(re.search(r"constexpr int kTileE = (\d+);", src).group(1))
    r4 = eval(re.search(r"constexpr int kR4 = ([^;]+);", src).group(1).replace("kTileE", str(te)))
    r8 = eval(re.search(r"constexpr int kR8 = ([^;]+);", src).group(1).replace("kTileE", str(te)))
    return te, r4, r8


def window(o, n, z):
    lo = (o * z) & ~15
    hi = ((o + n) * z + 15) & ~15
    return lo, hi - lo


def check_size(N, te, r4, r8):
    ntiles = (N + te - 1) // te
    for t in range(ntiles):
        s = t * te
        cnt = min(te, N - s)
        of = s - 1 if s > 0 else 0
        end = min(s + cnt + 1, N)
        nf, ngax = end - of, end - s
        # (first element, count, element size, region bytes, array length in elements)
        arrays = {"flags": (s, cnt, 4, r4, N), "F": (of, nf, 4, r4, N), "gax": (s, ngax, 4, r4, N),
                  "V": (s, cnt, 8, r8, N), "cdt": (s, cnt, 4, r4, N), "cls": (s, cnt, 4, r4, N),
                  "m": (s, cnt, 4, r4, 3 * N), "h": (N + s, cnt, 4, r4, 3 * N),
                  "n": (2 * N + s, cnt, 4, r4, 3 * N)}
        for name, (o, n, z, region, alen) in arrays.items():
            lo, nb = window(o, n, z)
            assert lo % 16 == 0 and nb % 16 == 0, (N, t, name)
            assert nb <= region, (N, t, name, nb, region)
            assert lo + nb <= (alen * z + 15) // 16 * 16, (N, t, name)
            assert lo <= o * z and (o + n) * z <= lo + nb, (N, t, name)
        for j in {s, s + 1, s + cnt - 2, s + cnt - 1} & set(range(s, s + cnt)):
            jm = j - 1 if j > 0 else j
            jp = j + 1 if j + 1 < N else j
            assert of <= jm and jp < of + nf, (N, t, j)      # F and its halo
            assert s <= j and jp < s + ngax, (N, t, j)       # conductances and theirs


def test_tile_windows():
    te, r4, r8 = constants()
    rng = random.Random(7)
    sizes = list(range(1, 3 * te + 40)) + [rng.randrange(1, 3_000_000) for _ in range(60)]
    for N in sizes:
        check_size(N, te, r4, r8)
