"""porelb_gb300: GB300-native sparse-lattice D3Q19 BGK solver (porelb's hot
path) behind a C ABI (include/porelb_gpu.h)."""
from ._lib import NODE_DTYPE, NB_DTYPE, Q, LIB_PATH  # noqa: F401
from .api import (PorelbError, Simulation, auto_ordering, build_table,  # noqa: F401
                  check_table, read_vbin, sphere_pack, sphere_pack_device,
                  write_vbin)
