"""GB300-native OpenMEEG symmetric-BEM forward path.

The compute path is libomg_gb300.so (hand-written sm_103a CUDA behind a C
ABI, ``include/openmeeg_gb300.h``); this package is its Python face.
"""
import importlib

__version__ = "0.1.0"

_API_NAMES = {"Context", "Geometry", "Integrator", "HeadMat", "HeadMatPacked", "DipSourceMat", "Head2EEGMat",
              "Head2MEGMat", "DipSource2MEGMat", "Solver", "GainEEG", "GainMEG", "GainEEGadjoint", "GainMEGadjoint",
              "GainEEGMEGadjoint", "forward_gain", "BatchForward", "SurfSourceMat", "SurfSource2MEGMat", "Surf2VolMat",
              "DipSource2InternalPotMat", "EITSourceMat", "OMGError",
              "kernel_launches"}


def __getattr__(name):
    # The torch-backed API is imported lazily so that numpy-only users
    # (file IO, synthetic heads) do not pay for importing torch.
    if name in _API_NAMES:
        return getattr(importlib.import_module(".api", __name__), name)
    raise AttributeError(name)
