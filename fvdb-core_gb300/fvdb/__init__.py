"""fvdb_gb300: fVDB's sparse 3-D convolution path rebuilt for GB300 (sm_103a).

Drop-in names of the reference package for this path: GridBatch, JaggedTensor,
SparseConvPackInfo, ConvPackBackend and fvdb.nn.{SparseConv3d, VDBTensor}.
"""

from . import _lib
from .grid_batch import GridBatch
from .jagged_tensor import JaggedTensor, jcat
from .sparse_conv_pack_info import ConvPackBackend, SparseConvPackInfo

_lib.load()

from . import nn  # noqa: E402

__version__ = "0.1.0"
__all__ = ["GridBatch", "JaggedTensor", "jcat", "SparseConvPackInfo", "ConvPackBackend", "nn"]
