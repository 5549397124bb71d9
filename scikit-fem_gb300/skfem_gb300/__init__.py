"""skfem_gb300: scikit-fem's cell assembly on a GB300 GPU (sm_103a).

Drop-in for ``BilinearForm.assemble`` / ``LinearForm.assemble`` on a
``CellBasis``: same API, same scipy CSR / numpy results, computed by
hand-written FP64 CUDA kernels through the C ABI in include/skfem_gb300.h.
"""

from .mesh import Mesh, MeshTri, MeshTri1, MeshTet, MeshTet1, MeshHex, MeshHex1  # noqa: F401
from .element import (Element, ElementH1, ElementTriP1, ElementTriP2, ElementTetP1,  # noqa: F401
                      ElementTetP2, ElementHex1, ElementVector)
from .quadrature import get_quadrature  # noqa: F401
from .dofs import Dofs  # noqa: F401
from .basis import Basis, CellBasis, FacetBasis  # noqa: F401
from .form import Form, BilinearForm, LinearForm, Functional, asm, ElementField  # noqa: F401
from .coo import COOData  # noqa: F401
from .field import DiscreteField  # noqa: F401
from . import helpers, models  # noqa: F401

__version__ = "0.1.0"


def build(force=False):
    """Compile the CUDA library in-tree (sm_103a)."""
    from . import _build
    return _build.build(force=force)


def lib():
    from . import _native
    return _native.lib()
