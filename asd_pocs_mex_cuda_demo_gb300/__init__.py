"""GB300-native (sm_103a) ASD-POCS hot path behind the reference's interface.

Entry points mirror the reference (imagereconstruction/ASD_POCS_mex_cuda_demo):

* ``Ax_cone_gpu`` / ``Atx_cone_gpu``   -- src/AxAtx mex gateways
* ``imgTVGradMin`` / ``imgTVGradMin3D`` -- src/tvmin mex functions
* ``ASD_POCS_cuda`` / ``SART_cuda_inline`` -- utilities/*.m drivers
* ``Plan`` -- batched, device-resident reconstructions (CUDA graphs), the
  instances of one batch free to differ in every size; ``plan_layout`` shows
  how a batch would run (its groups and streams) without a GPU
* ``Server`` -- serving queue: jobs submitted at any time, continuously
  batched on the device

All compute goes through the C ABI in ``lib/libasdpocs_gb300.so``
(declared in include/asdpocs_gb300.h); there is no CPU fallback.
"""
from ._lib import AsdpocsError, load  # noqa: F401
from .asdpocs import ASD_POCS_cuda, Plan, SART_cuda_inline, plan_layout  # noqa: F401
from .serve import Server  # noqa: F401
from .mex import (Atx_cone_gpu, Atx_cone_mf_gpu_new, Ax_cone_gpu,  # noqa: F401
                  Ax_cone_mf_gpu_new, Ax_siddon_mf_gpu, MexError, adjoint_check,
                  imgTVGradMin, imgTVGradMin3D)

__all__ = ["Ax_cone_gpu", "Atx_cone_gpu", "imgTVGradMin", "imgTVGradMin3D",
           "ASD_POCS_cuda", "SART_cuda_inline", "Plan", "Server", "Ax_cone_mf_gpu_new",
           "Atx_cone_mf_gpu_new", "Ax_siddon_mf_gpu", "MexError", "AsdpocsError", "load",
           "adjoint_check", "plan_layout"]
