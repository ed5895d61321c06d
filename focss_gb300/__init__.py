"""focss_gb300: GB300-native (sm_103a) split-step Fourier propagation, digital
back-propagation and perturbation equalization behind focss's API.

All compute runs in libfocss_gpu.so (hand-written CUDA, C ABI in
include/focss_gpu.h); this package is the host-side mirror of the reference's
C++ classes.
"""
from ._lib import FocssError, lib, LIB_PATH  # noqa: F401
from .api import (  # noqa: F401
    Amplifier, Context, Domain, Fiber, Field, SSFM, backward_propagation, cd_compensation,
    db_to_linear, db_to_natural, dbm_to_watts, disp_to_beta2, forward_propagation, launch_count,
    LIGHT_SPEED, MATH_PI, PLANCK, AMP_NONE, SPLIT_SINGLE_CTA, STAGING_BULK, STAGING_LOADS, STAGING_TMA, autotune, set_fft_split,
    set_pass_staging, set_row_staging, span_loop,
)
from . import dsp  # noqa: F401,E402
from .dsp import PhaseShiftEqualizer, ScalarEqualizer  # noqa: F401,E402
from .wdm_ppe import WdmPPE  # noqa: F401,E402
