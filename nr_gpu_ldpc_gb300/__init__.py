"""nr_gpu_ldpc_gb300 -- GB300-native 5G NR / QC-LDPC min-sum decoding.

* ``codes``    base graphs, lifting sizes, ``setup_ldpc`` (host logic, no GPU)
* ``Decoder``  the GPU decoder over the C-ABI library ``libnrldpc_gb300.so``
* ``build``    compiles that library (nvcc, sm_103a)

Importing this package needs no GPU; constructing a ``Decoder`` loads the
CUDA library and fails loudly if it is missing or no GPU is present.
"""
from . import codes  # noqa: F401
from .codes import LdpcParams, noise_sigma, setup_ldpc  # noqa: F401


def __getattr__(name):
    if name == "Decoder":
        from .decoder import Decoder
        return Decoder
    if name == "Trainer":
        from .learned import Trainer
        return Trainer
    raise AttributeError(name)
