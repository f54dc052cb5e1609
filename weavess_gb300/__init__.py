"""GB300-native implementation of the WEAVESS hot path: NN-Descent graph
construction, RNG / alpha pruning and batched greedy beam search, behind a C
ABI (include/weavess_gpu.h) with hand-written sm_103a kernels."""
from .index import Context  # noqa: F401
