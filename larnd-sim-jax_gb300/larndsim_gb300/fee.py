"""Front-end helpers (reference: src/larndsim/fee_jax.py)."""

from __future__ import annotations

import numpy as np
import torch

from .sim import (average_hit_values, get_adc_values, get_adc_values_average_noise_vmap,  # noqa: F401
                  get_average_hit_values)


def digitize(params, integral_list):
    """ADC counts from integrated charge, continuous (fee_jax.py:55-71)."""
    x = torch.as_tensor(integral_list, dtype=torch.float32)
    pre = (x * np.float32(params.GAIN) + np.float32(params.V_PEDESTAL)) - np.float32(params.V_CM)
    out = (torch.clamp(pre, min=0.0) * np.float32(params.ADC_COUNTS)) / np.float32(params.V_REF - params.V_CM)
    return torch.clamp(out, max=float(np.float32(params.ADC_COUNTS)))
