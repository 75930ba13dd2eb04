"""GB300 (sm_103a) implementation of SuLi-IC's per-time-step hot path."""
from ._abi import SuliParams, SuliDiag, default_params, field_shape, field_bounds, FIELDS  # noqa: F401
