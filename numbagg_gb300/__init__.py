"""numbagg_gb300: numbagg's scan and reduction hot path on a GB300 GPU.

Drop-in replacements, same names and keywords, for numbagg's moving-window,
exponentially weighted, fill, labelled-reduction and static aggregation functions.
Inputs may be torch CUDA tensors (results stay on the device) or numpy arrays / CPU
tensors (copied to the current CUDA device and back).  The compute is hand-written sm_103a CUDA behind
a C ABI (``include/numbagg_gb300.h``); there is no CPU fallback.
"""

from .aggregate import (
    allnan,
    anynan,
    count,
    nanargmax,
    nanargmin,
    nancount,
    nanmax,
    nanmean,
    nanmin,
    nanstd,
    nansum,
    nanvar,
)
from .funcs import bfill, ffill, nancorrmatrix, nancovmatrix
from .grouped import (
    group_nanall,
    group_nanany,
    group_nanargmax,
    group_nanargmin,
    group_nancount,
    group_nanfirst,
    group_nanlast,
    group_nanmax,
    group_nanmean,
    group_nanmin,
    group_nanprod,
    group_nanstd,
    group_nansum,
    group_nansum_of_squares,
    group_nanvar,
)
from .moving import move_corr, move_cov, move_mean, move_std, move_sum, move_var
from .moving_exp import (
    move_exp_nancorr,
    move_exp_nancount,
    move_exp_nancov,
    move_exp_nanmean,
    move_exp_nanstd,
    move_exp_nansum,
    move_exp_nanvar,
)
from .moving_matrix import move_corrmatrix, move_covmatrix, move_exp_nancorrmatrix, move_exp_nancovmatrix
from . import ragged  # noqa: E402  (ragged batches: an extension)

__version__ = "1.0.0"

# category lists, as numbagg/__init__.py:64-127 (restricted to this package's path;
# nanmedian / nanquantile are not built)
AGGREGATION_FUNCS = [
    allnan,
    anynan,
    count,
    nanargmax,
    nanargmin,
    nancount,
    nanmax,
    nanmean,
    nanmin,
    nanstd,
    nansum,
    nanvar,
]
GROUPED_FUNCS = [
    group_nanall,
    group_nanany,
    group_nanargmax,
    group_nanargmin,
    group_nancount,
    group_nanfirst,
    group_nanlast,
    group_nanmax,
    group_nanmean,
    group_nanmin,
    group_nanprod,
    group_nanstd,
    group_nansum,
    group_nansum_of_squares,
    group_nanvar,
]
MOVE_EXP_FUNCS = [
    move_exp_nancorr,
    move_exp_nancount,
    move_exp_nancov,
    move_exp_nanmean,
    move_exp_nanstd,
    move_exp_nansum,
    move_exp_nanvar,
]
MOVE_EXP_MATRIX_FUNCS = [move_exp_nancorrmatrix, move_exp_nancovmatrix]
MOVE_FUNCS = [move_corr, move_cov, move_mean, move_corrmatrix, move_covmatrix, move_std, move_sum, move_var]
MATRIX_FUNCS = [nancorrmatrix, nancovmatrix]
OTHER_FUNCS = [bfill, ffill]

__all__ = [
    "AGGREGATION_FUNCS",
    "GROUPED_FUNCS",
    "MATRIX_FUNCS",
    "MOVE_EXP_FUNCS",
    "MOVE_EXP_MATRIX_FUNCS",
    "MOVE_FUNCS",
    "OTHER_FUNCS",
    "allnan",
    "anynan",
    "bfill",
    "count",
    "ffill",
    "group_nanall",
    "group_nanany",
    "group_nanargmax",
    "group_nanargmin",
    "group_nancount",
    "group_nanfirst",
    "group_nanlast",
    "group_nanmax",
    "group_nanmean",
    "group_nanmin",
    "group_nanprod",
    "group_nanstd",
    "group_nansum",
    "group_nansum_of_squares",
    "group_nanvar",
    "move_corr",
    "move_corrmatrix",
    "move_cov",
    "move_covmatrix",
    "move_exp_nancorr",
    "move_exp_nancorrmatrix",
    "move_exp_nancount",
    "move_exp_nancov",
    "move_exp_nancovmatrix",
    "move_exp_nanmean",
    "move_exp_nanstd",
    "move_exp_nansum",
    "move_exp_nanvar",
    "move_mean",
    "move_std",
    "move_sum",
    "move_var",
    "nanargmax",
    "nanargmin",
    "nancorrmatrix",
    "nancount",
    "nancovmatrix",
    "nanmax",
    "nanmean",
    "nanmin",
    "nanstd",
    "nansum",
    "nanvar",
]
