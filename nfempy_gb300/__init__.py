"""nfempy_gb300 - GB300-native finite-element assembly-and-solve hot path.

Host API mirroring nfempy (ProductSpace, WeakForm, SequentialAssembler) over a
C-ABI CUDA library (libnfem_gb300.so, include/nfem_gb300.h) compiled for
sm_103a.  Build with `nfempy_gb300.build.build()`.
"""
from . import _lib  # noqa: F401
from .assembly import (CSRMatrix, LaplaceDualWeakForm, LaplaceDualWeakFormBCDirichlet,  # noqa: F401
                       LCEDualWeakForm, LCEDualWeakFormBCDirichlet, LCEScaledRieszMapWeakForm, LEPrimalWeakForm, LEPrimalWeakFormBCDirichlet, LEDualWeakForm, LEDualWeakFormBCDirichlet, LERieszMapWeakForm,
                       SequentialAssembler, WeakForm, div_error, div_norm, div_scaled_error, l2_error, l2_norm)
from .spaces import DiscreteSpace, Mesh, ProductSpace  # noqa: F401

__all__ = ["CSRMatrix", "LaplaceDualWeakForm", "LaplaceDualWeakFormBCDirichlet", "LCEDualWeakForm",
           "LCEDualWeakFormBCDirichlet", "LCEScaledRieszMapWeakForm", "LEPrimalWeakForm", "LEPrimalWeakFormBCDirichlet", "LEDualWeakForm", "LEDualWeakFormBCDirichlet", "LERieszMapWeakForm", "SequentialAssembler",
           "WeakForm", "l2_error", "l2_norm", "div_error", "div_norm", "div_scaled_error", "DiscreteSpace", "Mesh",
           "ProductSpace"]
