"""jubik_gb300 -- GB300 (sm_103a) implementation of J-UBIK's spatially-variant
X-ray instrument response (patch PSF convolution, exposure, readout) and its
Poisson likelihood, with hand-written adjoints.

The public names mirror ``jubik`` (``jubik/__init__.py:40,59``) for this path:
``Domain``, ``slice_patches``, ``linpatch_convolve``, ``convolve``,
``build_exposure_function``, ``build_readout_function``, ``coord_center``,
plus the likelihood (``Poissonian``) and instrument builders.
"""
from __future__ import annotations

import numpy as np

from ._lib import JubikError, JubikStateError, JubikUnsupported
from .batch import ProblemBatch
from . import diagnostics, minimization, psf, sampling
from .convolve import (Domain, _bilinear_weights, convolve, integrate, linpatch_convolve,
                       slice_patches, slice_patches_adjoint)
from .instruments import Response, build_psf_op, build_response
from .likelihood import ModelPoissonian, Poissonian, ResponsePoissonian
from .plan import ResponsePlan
from .response import Vector, build_exposure_function, build_readout_function

__version__ = "0.1.0"


def coord_center(side_length, side_n):
    """Flat indices of the n^2 patch centres, in slice_patches order
    (``jubik/utils.py:185-207``)."""
    tdx = tdy = side_length // side_n
    xc = np.arange(tdx // 2, tdx * side_n, tdx)
    yc = np.arange(tdy // 2, tdy * side_n, tdy)
    co = np.array(np.meshgrid(xc, yc)).reshape(2, -1)
    return np.ravel_multi_index(co, [side_length, side_length])


__all__ = [
    "Domain", "slice_patches", "slice_patches_adjoint", "linpatch_convolve", "convolve",
    "integrate", "_bilinear_weights", "build_exposure_function", "build_readout_function",
    "coord_center", "Vector", "Poissonian", "ResponsePoissonian", "ModelPoissonian",
    "Response", "build_response", "build_psf_op", "ResponsePlan", "JubikError",
    "JubikUnsupported", "JubikStateError", "ProblemBatch",
]
