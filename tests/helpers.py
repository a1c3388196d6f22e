"""Shared helpers for the tests: descriptor builders from golden fixtures."""
import numpy as np

from oracle.oracle import CheckerDesc, SpaceDesc


def space_of(g):
    return SpaceDesc(int(g["space_kind"]), int(g["dim"]), g["low"], g["high"], float(g["link_length"]),
                     float(g["lvs_fraction"]), int(g["factor"]))


def checker_of(g):
    return CheckerDesc(int(g["checker_kind"]), g["obstacles"], g["dh"] if g["dh"].size else None,
                       int(g["spheres_per_link"]), float(g["sphere_radius"]))


def same_bits(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return np.array_equal(a.view(np.uint64) if a.dtype == np.float64 else a, b.view(np.uint64)
                              if b.dtype == np.float64 else b) or np.array_equal(a, b, equal_nan=True) and \
            np.array_equal(np.signbit(a), np.signbit(b))
    return np.array_equal(a, b)
