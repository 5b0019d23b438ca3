"""genesis_gb300: GB300-native MLS-MPM substep behind Genesis's scene / entity API.

    import genesis_gb300 as gs
    gs.init(backend=gs.gpu)
    scene = gs.Scene(sim_options=gs.options.SimOptions(dt=2e-4),
                     mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)))
    cube = scene.add_entity(material=gs.materials.MPM.Elastic(), morph=gs.morphs.Box(pos=(.5, .5, .4), size=(.2,) * 3))
    scene.build()
    scene.step()
    state = cube.get_state()

Every substep runs in libgbmpm.so (hand-written sm_103a CUDA).  There is no CPU backend
and no fallback: gs.init(backend=gs.cpu) and a missing library both raise.
"""

from __future__ import annotations

import random as _random
import types as _types

import numpy as np

from . import materials as _materials_mod
from . import force_fields, morphs
from . import options as _options_mod
from .entity import ACTIVE, INACTIVE
from .exceptions import GenesisException
from .scene import Scene

__version__ = "0.1.0"

gpu = "gpu"
cuda = "cuda"
cpu = "cpu"

EPS = float(np.finfo(np.float32).eps)
_initialized = False
backend = None
device = None
precision = "32"


class options(_types.SimpleNamespace):
    SimOptions = _options_mod.SimOptions
    MPMOptions = _options_mod.MPMOptions
    LegacyCouplerOptions = _options_mod.LegacyCouplerOptions
    ToolOptions = _options_mod.ToolOptions
    ViewerOptions = _options_mod.ViewerOptions
    VisOptions = _options_mod.VisOptions
    ProfilingOptions = _options_mod.ProfilingOptions
    morphs = morphs


class materials(_types.SimpleNamespace):
    MPM = _materials_mod.MPM
    Tool = _materials_mod.Tool


class surfaces(_types.SimpleNamespace):
    class Default:
        def __init__(self, **kw):
            self.__dict__.update(kw)

    Rough = Smooth = Plastic = Glass = Water = Default


def init(seed=None, precision="32", debug=False, eps=1e-15, backend=None, logging_level=None, **kwargs):
    """genesis/__init__.py:57-293 for the MPM path: CUDA backend, fp32, EPS, seeding."""
    global _initialized, EPS, device
    import genesis_gb300 as _self
    import torch

    if backend is None:
        backend = gpu
    if backend not in (gpu, cuda):
        raise GenesisException(
            f"backend {backend!r} is not supported: this MPM path runs only on the CUDA GPU (no CPU fallback)."
        )
    if str(precision) != "32":
        raise GenesisException("Only precision='32' is supported by the GB300 MPM kernels.")
    if not torch.cuda.is_available():
        raise GenesisException("No CUDA device available: this MPM path has no CPU fallback.")
    EPS = max(float(eps), float(np.finfo(np.float32).eps))  # genesis/__init__.py:229
    if seed is not None:  # utils/misc.py:154-161
        _random.seed(seed)
        np.random.seed(seed)
        torch.manual_seed(seed)
    _self.backend = backend
    _self.precision = "32"
    device = torch.device("cuda", torch.cuda.current_device())
    _initialized = True


def destroy():
    global _initialized
    _initialized = False


def build_library(force: bool = False) -> str:
    """Compile libgbmpm.so in-tree (sm_103a)."""
    from .build import build

    return build(force=force)


__all__ = [
    "init",
    "destroy",
    "Scene",
    "options",
    "materials",
    "morphs",
    "surfaces",
    "GenesisException",
    "ACTIVE",
    "INACTIVE",
    "gpu",
    "cuda",
    "cpu",
]
