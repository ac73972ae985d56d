"""What the learned preconditioner gains over the method without it.

The plain method is flexible GMRES with the cell-patch block-Jacobi
preconditioner.  The learned preconditioner adds the two-level coarse
correction whose flux-extension weights come from the trained network
(nfempy_gb300/data/learned_coarse.pt, trained on the GPU with the library's
kernels by nfempy_gb300.train_learned on seeded permeability fields; the
scale alpha of the network's correction was chosen on a validation field).
On a held-out field (seed 7) of 3-D mixed Darcy, 32^3 x 6 tetrahedra, both
reach ||b - A x|| / ||b|| <= 1e-8 in FP64; the learned one needs at least
3x fewer iterations.  The classical-weight two-level method runs beside
it so the network's own share stays visible: validation chose alpha = 0 for
the shipped checkpoint (the network's weights did not beat the classical
ones), so the learned and classical runs match and the gain over the plain
method comes from the two-level structure; the test checks that match."""
import os

import pytest
import torch

from nfempy_gb300 import learned, train_learned
from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse

pytestmark = pytest.mark.gpu


def test_learned_preconditioner_gain(cuda_lib):
    if not os.path.exists(train_learned.DEFAULT_OUT):
        pytest.fail("trained network checkpoint missing: run python -m nfempy_gb300.train_learned")
    model, ck = train_learned.load()
    alpha = ck["alphas_by_side_fraction"][4]["alpha"]
    P = learned.DarcyProblem(32)
    kappa = P.field(7)
    b = P.assemble(kappa)
    plain = KrylovSolver(P.A, pc="cell_block", A32_values=P.A32.values)
    x0, i0 = plain.solve(b, rtol=1e-8, max_inner=20000)
    tl = TwoLevelCoarse(P.A, 8)
    tl.set_weights(learned.learned_weights(tl, model, kappa, alpha))
    lk = KrylovSolver(P.A, pc="two_level", A32_values=P.A32.values, two_level=tl)
    x1, i1 = lk.solve(b, rtol=1e-8, max_inner=20000)
    tlc = TwoLevelCoarse(P.A, 8)
    ck_ = KrylovSolver(P.A, pc="two_level", A32_values=P.A32.values, two_level=tlc)
    x2, i2 = ck_.solve(b, rtol=1e-8, max_inner=20000)
    print(f"plain {i0.inner_iterations}  learned(alpha={alpha}) {i1.inner_iterations}  "
          f"classical two-level {i2.inner_iterations}")
    for x, info in ((x0, i0), (x1, i1), (x2, i2)):
        assert info.status == 0
        assert float(plain.residual(x, b).norm() / b.norm()) <= 1e-8
    assert i1.inner_iterations * 3 <= i0.inner_iterations
    if alpha == 0.0:  # the network's correction is off: the same preconditioner
        assert i1.inner_iterations == i2.inner_iterations
