"""mojovec_gb300: MojoVec's vector-query and index-training hot path on one
NVIDIA GB300 (sm_103a).

The compute lives in libmojovec_gpu.so (hand-written CUDA behind the C ABI
in include/mojovec_gpu.h). This package is the host-side mirror of the
reference's interfaces over that ABI: IndexIVFPQ, IndexFlat, IndexFlatSQ8,
KMeans, ProductQuantizer and the managed IVFPQCollection.
"""

from ._lib import (  # noqa: F401
    FORM_FAST,
    FORM_PLAIN,
    METRIC_IP,
    METRIC_L2,
    MojoVecGPUError,
)
from .collection import IVFPQCollection  # noqa: F401
from .index import (  # noqa: F401
    Context,
    IndexFlat,
    IndexFlatSQ8,
    IndexIVFFlat,
    IndexIVFPQ,
    IVFPQBatchPlan,
    KMeans,
    Server,
    distance_matrix,
    ProductQuantizer,
    normalize,
    sq8_encode,
)

__version__ = "0.1.0"
