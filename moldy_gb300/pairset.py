"""Canonical form of an evaluated site-pair set.

Moldy evaluates each site pair once per (reference cell, neighbour-cell
offset) combination (src/force.c:856-967).  A pair is identified by the two
site indices and the periodic image of the second site, encoded as in the
reference's pbctrans table (src/force.c:1263-1272):
``image = 9*(nx+1) + 3*(ny+1) + (nz+1)`` for r = x_j + h.(nx,ny,nz) - x_i.

Reversing a pair negates the image (``26 - image``), so a canonical key
orients every pair with i < j (for i == j, the smaller image code), and packs
it as ``(i << 37) | (j << 5) | image``.
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def canonical_keys(i, j, image) -> np.ndarray:
    """Sorted canonical uint64 keys of pairs given as (i, j, image) arrays."""
    i = np.asarray(i, np.int64)
    j = np.asarray(j, np.int64)
    k = np.asarray(image, np.int64)
    neg = 26 - k
    swap = (i > j) | ((i == j) & (k > neg))
    a = np.where(swap, j, i)
    b = np.where(swap, i, j)
    kk = np.where(swap, neg, k)
    return np.sort(((a << 37) | (b << 5) | kk).astype(np.uint64))


def keys_from_triplets(p) -> np.ndarray:
    p = np.asarray(p)
    return canonical_keys(p[:, 0], p[:, 1], p[:, 2])


def digest(keys) -> tuple:
    """Order-independent digest of a key set: (count, sum of mixed keys mod
    2^64).  A splitmix64 finaliser spreads each key before summing."""
    z = np.asarray(keys, np.uint64).copy()
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
        s = int(np.sum(z, dtype=np.uint64))
    return int(len(keys)), s
