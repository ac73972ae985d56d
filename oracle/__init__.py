"""CPU oracle for the nfempy assembly-and-solve hot path (TEST INFRASTRUCTURE).

This package is a plain FP64 numpy restatement of the reference's algorithms.
It exists only to check the GPU product: `tests/`, `__graft_entry__.smoke()`
and the CPU-baseline / reference legs of `bench.py` may import it; the product
package `nfempy_gb300` never does.

Module map (each function cites the reference file:line it restates):

  quadrature.py  collapsed Gauss-Jacobi rules     (src/spaces/product_space.py:23-50)
  elements.py    P0/P1/P2 Lagrange, RT1 tables    (src/basis/finite_element.py:156-186)
  mesh_gen.py    synthetic gmsh-like meshes       (src/mesh/mesh.py:239-339 input format)
  topology.py    entity ids, first-appearance DoF maps, orientation
                                                  (src/mesh/mesh.py, src/spaces/dof_map.py,
                                                   src/basis/permute_and_transform.py)
  geometry.py    affine map, |det J|, pseudo-inverse (src/geometry/mapping.py:23-55)
  forms.py       weak-form element matrices       (src/weak_forms/*.py)
  assembly.py    element-clique CSR pattern and scatter (src/assembly/ScatterFormData.py:5-25)
  solve.py       direct solve and L2 error norms  (src/postprocess/l2_error_post_processor.py:7-63)

Parity status: DoF maps, sparsity patterns, orientation flags, mapping
(det/pseudo-inverse) and the oriented basis tabulation are pinned against the
reference's own code run on the same meshes (fixtures in tests/golden/, made by
tests/golden/make_golden.py).  The RT1 normalisation and reference-normal sign
convention follow basix's published element definition and are NOT pinned by
any reference test or fixture ("parity unpinned" for RT scale/sign).
"""
