"""Shared test cases: meshes and field layouts matching tests/golden/*.npz."""
import os

import numpy as np

from oracle import mesh_gen

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

DARCY = [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)]
CASES = {
    "darcy2d_n4": (lambda: mesh_gen.square(4), DARCY),
    "darcy3d_n2": (lambda: mesh_gen.cube(2), DARCY),
    "elast3d_n2": (lambda: mesh_gen.cube(2), [("u", "P", 2, 3, False)]),
    "elast2d_n3": (lambda: mesh_gen.square(3), [("u", "P", 2, 2, False)]),
    "cosserat3d_n1": (lambda: mesh_gen.cube(1), [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False),
                                                 ("u", "P", 0, 3, True), ("t", "P", 0, 3, True)]),
}


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def to_product_fields(fields):
    """Oracle family names -> reference names ('P' -> 'Lagrange')."""
    return [(n, "Lagrange" if f == "P" else f, k, nc, d) for n, f, k, nc, d in fields]
