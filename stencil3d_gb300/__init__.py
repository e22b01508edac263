"""stencil3d_gb300: the stencil3d hot path (2/7/13/25-point 3-D cross
stencils over the u/v/s fields) as hand-written CUDA kernels for one GB300
(sm_103a), behind a C ABI (include/st3d.h) with a hstencil3d-compatible C++
driver and this Python binding.
"""
from .api import (  # noqa: F401
    Grid, Stencil, Batch, St3dError, PinnedArray, default_opts, plan, device_info, ricker,
    iterate_gb300, init_arrays, check, lib, last_error,
    MODE_REF, MODE_WAVE, F32, F64, F16, BF16, F16_HILO, F16_HL,
    KERNEL_AUTO, KERNEL_SIMPLE, KERNEL_TMA, KERNEL_MMA, FIELD_U, FIELD_V, FIELD_S,
    FILL_CONST, FILL_UNIFORM, FILL_BLOBS,
    BATCH_SEQUENTIAL, BATCH_PERSISTENT, BATCH_GRAPH,
)
