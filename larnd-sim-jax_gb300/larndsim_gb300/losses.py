"""Loss-side helpers (reference: src/larndsim/losses_jax.py)."""

from __future__ import annotations

import numpy as np
import torch


def adc2charge(dw, params):
    """Charge in ke- from ADC counts (losses_jax.py:380-383)."""
    x = torch.as_tensor(dw, dtype=torch.float32)
    return ((((x / np.float32(params.ADC_COUNTS)) * np.float32(params.V_REF - params.V_CM))
             + np.float32(params.V_CM)) - np.float32(params.V_PEDESTAL)) / np.float32(params.GAIN) * np.float32(1e-3)
