"""Shared test cases: meshes and field layouts matching tests/golden/*.npz."""
import os

import numpy as np

from oracle import mesh_gen

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

DARCY = [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)]
def golden_mesh(name):
    """The gmsh mesh stored in a fixture (read from the reference's .msh by
    tests/golden/make_golden.py)."""
    g = golden(name)
    blocks = []
    i = 0
    while f"block{i}_type" in g:
        blocks.append((str(g[f"block{i}_type"]), g[f"block{i}_conn"], g[f"block{i}_phys"]))
        i += 1
    return {"dim": int(g["mesh_dim"]), "points": g["points"], "blocks": blocks}


LE_FIELDS = [("s", "RT", 1, 3, False), ("u", "P", 0, 3, True), ("t", "P", 0, 3, True)]
COSSERAT_FIELDS = [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False), ("u", "P", 0, 3, True), ("t", "P", 0, 3, True)]
CASES = {
    "darcy2d_n4": (lambda: mesh_gen.square(4), DARCY),
    "darcy3d_n2": (lambda: mesh_gen.cube(2), DARCY),
    "elast3d_n2": (lambda: mesh_gen.cube(2), [("u", "P", 2, 3, False)]),
    "elast2d_n3": (lambda: mesh_gen.square(3), [("u", "P", 2, 2, False)]),
    "cosserat3d_n1": (lambda: mesh_gen.cube(1), [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False),
                                                 ("u", "P", 0, 3, True), ("t", "P", 0, 3, True)]),
    "darcy3d_msh0": (lambda: golden_mesh("darcy3d_msh0"), DARCY),
    "cosserat3d_msh0": (lambda: golden_mesh("cosserat3d_msh0"), COSSERAT_FIELDS),
    "le3d_n1": (lambda: mesh_gen.cube(1), LE_FIELDS),
    "le3d_msh0": (lambda: golden_mesh("le3d_msh0"), LE_FIELDS),
}


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def to_product_fields(fields):
    """Oracle family names -> reference names ('P' -> 'Lagrange')."""
    return [(n, "Lagrange" if f == "P" else f, k, nc, d) for n, f, k, nc, d in fields]


# Coefficient functions of the element-form fixtures.  The reference's weak
# forms call them on quadrature-point coordinates: kappa point by point
# (laplace_dual_weak_form.py:71), the others on arrays (le_primal_weak_form.py:
# 37-39, lce_dual_weak_form.py:476-489).  Every Cosserat parameter differs so
# that each term of the form is pinned on its own.
def _const(v):
    return lambda x, y, z: np.full(np.shape(x), float(v))


COSSERAT_PARAMS = dict(lambda_s=1.3, mu_s=0.7, kappa_s=0.45, lambda_o=0.9, mu_o=1.1, kappa_o=0.35, l=0.8)
COSSERAT_RHS = (1.0, -2.0, 0.5, 0.3, 0.2, -0.4)


def cosserat_rhs(x, y, z):
    """A load that varies inside the cells (f_u then f_t, [6, N])."""
    return np.array([COSSERAT_RHS[0] + x, COSSERAT_RHS[1] + y * z, COSSERAT_RHS[2] + np.sin(np.pi * z),
                     COSSERAT_RHS[3] * x * y, COSSERAT_RHS[4] + 0.0 * x, COSSERAT_RHS[5] + y * y])


# the Riesz map of the scaled Cosserat form with a length scale that varies
# (its grad l . v term), constant material
RIESZ_FUNCTIONS = {**{k: _const(v) for k, v in COSSERAT_PARAMS.items() if k != "l"},
                   "l": lambda x, y, z: 0.8 + 0.3 * x - 0.1 * y * z,
                   "grad_l": lambda x, y, z: np.array([0.3 + 0.0 * x, -0.1 * z, -0.1 * y])}

# the mixed linear-elastic Riesz map (LERieszMapWeakForm): constant
# material; the reference reads "rhs" but the operator does not use it
LE_RIESZ_FUNCTIONS = {"lambda": _const(1.3), "mu": _const(0.7),
                      "rhs": lambda x, y, z: np.zeros((3,) + np.shape(x))}

FORM_FUNCTIONS = {
    "darcy": {
        "kappa": lambda x, y, z: 1.0 + 0.5 * x + 0.25 * y * y + 0.1 * z,
        "rhs": lambda x, y, z: np.array([np.sin(np.pi * x) * np.sin(np.pi * y) + z]),
    },
    "elast": {
        "lambda": lambda x, y, z: 1.0 + x + 0.0 * y,
        "mu": lambda x, y, z: 2.0 + y * z + 0.5 * x,
        "rhs": lambda x, y, z: np.array([x + 0.0 * y, 1.0 + 0.0 * x, z * z + y]),
    },
    "cosserat": {
        **{k: _const(v) for k, v in COSSERAT_PARAMS.items()},
        "rhs": cosserat_rhs,
    },
    # LEDualWeakForm: constant material (the device form takes one), a load
    # that varies inside the cells
    "le": {"lambda": _const(1.3), "mu": _const(0.7), "rhs": cosserat_rhs},
}

# coefficients the device forms take as they are: kappa, lambda and mu
# constant on each cell (here constant), the Darcy source sampled at the
# quadrature points, a constant elasticity load (the Cosserat case above
# already fits: constant material, a load the device integrates exactly)
FORM_FUNCTIONS_DEVICE = {
    "darcy": {
        "kappa": _const(2.5),
        "rhs": FORM_FUNCTIONS["darcy"]["rhs"],
    },
    "elast": {
        "lambda": _const(1.3),
        "mu": _const(0.8),
        "rhs": lambda x, y, z: np.array([1.0 + 0.0 * x, -0.5 + 0.0 * x, 0.25 + 0.0 * x]),
    },
}
