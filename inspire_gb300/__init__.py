"""GB300-native (sm_103a) ReinsPIRe online answer path.

The CUDA kernels and the C ABI live in libinspire_gb300.so (csrc/, built by
build.py); pir.py mirrors the reference PirServer API on top of that ABI.
"""
from .pir import (ENGINE_PLAIN, ENGINE_TENSOR, GadgetParams, InspireError,
                  PirParams, PirPreprocessedData, PirRequest, PirResponse,
                  PirServer, PreprocessMatrixPackOutput, RlweParams)

__all__ = ["ENGINE_PLAIN", "ENGINE_TENSOR", "GadgetParams", "InspireError",
           "PirParams", "PirPreprocessedData", "PirRequest", "PirResponse",
           "PirServer", "PreprocessMatrixPackOutput", "RlweParams"]
