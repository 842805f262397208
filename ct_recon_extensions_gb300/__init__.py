"""GB300-native (sm_103a) filtered-backprojection and projection hot path of
CT_RECON_EXTENSIONS.

* ``libctrecon_gb300.so`` -- CUDA kernels behind a C ABI (include/ctrecon_gb300.h)
* ``torch_ctrecon``       -- PyTorch front end mirroring the reference's
  tf_ctrecon.py functions, differentiable through the adjoint kernels
* ``synthetic``           -- seeded ellipse phantoms and analytic sinograms

Build the library with ``python -m ct_recon_extensions_gb300.build``.
"""
from ._lib import CtrError, CtrLibraryError, load  # noqa: F401

__version__ = "1.0.0"
