"""GB300 (sm_103a) implementation of GraAda3D's forward-modelling and
inversion hot path: prism sensitivity assembly, dense products with G, and
the Gauss-Newton + CG inversion, behind the C ABI of ``include/grada_gpu.h``.
"""
from .fwd import FIELD_BITS, FIELD_ORDER, Context, Fwd, field_mask, mask_fields  # noqa: F401
from ._lib import GradaError  # noqa: F401

__all__ = ["Context", "Fwd", "FIELD_BITS", "FIELD_ORDER", "field_mask", "mask_fields", "GradaError"]
