"""risltc_gb300: risltc's per-pixel many-light shading path (RIS over polygonal
lights with an LTC target, projected solid angle sampling, shadow rays, MIS)
as hand-written CUDA for GB300 (sm_103a) behind a C ABI (include/risltc.h)."""
from . import api, scenes  # noqa: F401
from .api import (Context, Scene, Model, RisltcError, settings, copy_settings, shade, shade_batch,  # noqa: F401
                  shade_host, trace_shadow, noise_constants, autotune, autotune_batch)
