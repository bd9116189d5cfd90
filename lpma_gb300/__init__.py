"""GB300-native LPMA: batched edge updates of a leveled packed memory array.

The compute path is the CUDA library lpma_gb300/_lpma.so (hand-written
sm_103a kernels behind the C ABI of include/lpma.h).  Importing the package
loads it and fails loudly when it has not been built.
"""
from . import _abi

_abi.load()

from .rpma import (Batcher, Lpma, LpmaError, default_config, destroy_rpma, gen_rmat_device, get_data_rpma,  # noqa: E402
                   gpma_config, gpma_key, init_csr_rpma, kernel_launches, pack_key, profile_enable, profile_report, sentinel_key,
                   shuffle_device, to_csr_rpma, update_rpma)

__all__ = ["Lpma", "Batcher", "LpmaError", "default_config", "gpma_config", "gpma_key", "init_csr_rpma", "update_rpma", "to_csr_rpma", "get_data_rpma",
           "destroy_rpma", "pack_key", "sentinel_key", "gen_rmat_device", "shuffle_device", "kernel_launches",
           "profile_enable", "profile_report"]
