"""GB300-native (sm_103a) implementation of larnd-sim-jax's simulate path.

Drop-in functions with the reference's names (src/larndsim/sim_jax.py,
consts_jax.py, fee_jax.py, losses_jax.py, optimize/strategies.py,
optimize/dataio.py, optimize/simulate.py's output records), backed by
hand-written CUDA kernels in ``liblsim.so`` (C ABI: include/lsim.h).
"""

from .consts import (Params, RecombinationMode, build_params_class, default_params, get_vdrift,  # noqa: F401
                     load_detector_properties)
from .sim import (average_hit_values, get_adc_values, get_adc_values_average_noise_vmap,  # noqa: F401
                  get_average_hit_values, load_lut, pad_size, prepare_lut, simulate_parametrized,
                  simulate_probabilistic, simulate_stochastic, simulate_wfs)
from .fee import digitize  # noqa: F401
from .losses import adc2charge, chamfer_3d, llhd_loss, mse_adc, nll_loss  # noqa: F401
from .dataio import DataLoader, TgtTracksDataset, TracksDataset, chop_tracks  # noqa: F401
from .detsim import (validate_event_ids_for_packing, validate_local_event_ids,  # noqa: F401
                     validate_packed_ids_for_decoding)
from .output import hit_records, write_hits_groups_npz, write_hits_h5, write_hits_npz  # noqa: F401

__all__ = [
    "Params", "RecombinationMode", "build_params_class", "default_params", "get_vdrift",
    "load_detector_properties", "get_adc_values", "load_lut", "pad_size", "prepare_lut",
    "simulate_parametrized", "simulate_stochastic", "simulate_wfs", "digitize", "adc2charge", "chop_tracks",
    "simulate_probabilistic", "get_adc_values_average_noise_vmap", "get_average_hit_values", "average_hit_values",
    "mse_adc", "nll_loss", "chamfer_3d", "llhd_loss", "hit_records", "write_hits_npz", "write_hits_h5", "write_hits_groups_npz",
    "TracksDataset", "TgtTracksDataset", "DataLoader", "validate_event_ids_for_packing",
    "validate_local_event_ids", "validate_packed_ids_for_decoding",
]
