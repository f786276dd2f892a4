"""ctgb -- GB300 (sm_103a) CT projector / backprojector library.

A from-scratch implementation of the hot path of CT-Research: Siddon
forward projectors (cone 3D, fan and parallel 2D), voxel-driven
backprojectors, FDK / FBP filtering and the SIRT(-TV) loops that call them.

* ``ctgb.ops``      -- the reference's MEX operators, same signatures (host arrays)
* ``ctgb.device``   -- plans over torch CUDA tensors (HBM-resident loops)
* ``ctgb.sirt``     -- SIRT / SIRT3D / SIRT-TV drivers
* ``ctgb.geometry`` -- scan geometries and the benchmark workloads
* ``ctgb.phantom``  -- seeded ellipse / ellipsoid phantoms
"""
from . import geometry, phantom  # noqa: F401

__version__ = "0.1.0"


def load():
    """Build if needed and load libctgb.so; returns the ctypes handle."""
    from . import _lib
    return _lib.load()
