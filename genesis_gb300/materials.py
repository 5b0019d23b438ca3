"""MPM materials with the reference's defaults and derived constants.

Mirrors genesis/engine/materials/MPM/{base,elastic,liquid,sand,snow,elasto_plastic,
muscle}.py.  The physics lives in the CUDA kernels; these classes carry parameters and
produce the C-ABI material record.
"""

from __future__ import annotations

import math
import re

from . import _lib
from .exceptions import GenesisException

_SAMPLER_PATTERN = re.compile(r"^pbs(-\d+)?$|^random$|^regular$")


class _MPMBase:
    """genesis/engine/materials/MPM/base.py:35-99."""

    _fields = ("E", "nu", "rho", "lam", "mu", "sampler")
    E = 1e6
    nu = 0.2
    rho = 1000.0
    lam = None
    mu = None
    # The reference defaults to 'pbs' on x86-64 Linux, which needs its prebuilt sampler binary
    # and falls back to 'random' when it fails (utils/particle.py:226-231); 'random' here.
    sampler = "random"
    _default_Jp = 1.0

    def __init__(self, **kw):
        fields = set()
        for cls in type(self).__mro__:
            fields |= set(getattr(cls, "_fields", ()))
        unknown = set(kw) - fields
        if unknown:
            raise GenesisException(f"Unrecognized attribute(s) for {type(self).__name__}: {sorted(unknown)}")
        self._all_fields = tuple(sorted(fields))
        for f in fields:
            setattr(self, f, kw.get(f, getattr(type(self), f)))
        if not (self.E > 0) or not (-1.0 < self.nu < 0.5) or not (self.rho > 0):
            raise GenesisException("Invalid E / nu / rho")
        if not isinstance(self.sampler, str) or not _SAMPLER_PATTERN.match(self.sampler):
            raise GenesisException("Input should be 'pbs', 'pbs-<seed>', 'random', or 'regular'")
        self.idx = None
        # base.py:77-83
        if self.mu is None:
            self.mu = self.E / (2.0 * (1.0 + self.nu))
        if self.lam is None:
            self.lam = self.E * self.nu / ((1.0 + self.nu) * (1.0 - 2.0 * self.nu))
        self._post_init()

    def _post_init(self) -> None:
        pass

    def __eq__(self, other) -> bool:
        return type(self) is type(other) and all(getattr(self, f) == getattr(other, f) for f in self._all_fields)

    def __hash__(self) -> int:
        return id(self)

    def __repr__(self) -> str:
        return f"MPM.{type(self).__name__}(" + ", ".join(f"{f}={getattr(self, f)!r}" for f in self._all_fields) + ")"

    # C-ABI record
    _type = _lib.MAT_ELASTIC

    def _flags(self) -> int:
        return 0

    def to_c(self, scene: int) -> _lib.MpmMaterial:
        m = _lib.MpmMaterial()
        m.type = self._type
        m.flags = self._flags()
        m.scene = scene
        m.mu = float(self.mu)
        m.lam = float(self.lam)
        m.rho = float(self.rho)
        m.default_Jp = float(self._default_Jp)
        m.friction_alpha = float(getattr(self, "alpha", 0.0))
        m.yield_lower = float(getattr(self, "yield_lower", 0.0))
        m.yield_higher = float(getattr(self, "yield_higher", 0.0))
        m.von_mises_yield_stress = float(getattr(self, "von_mises_yield_stress", 0.0))
        m.stiffness = float(getattr(self, "stiffness", 0.0))
        return m


class Elastic(_MPMBase):
    """elastic.py:12-60: E default 3e5, model 'corotation' | 'neohooken'."""

    _fields = ("model",)
    E = 3e5
    model = "corotation"
    _type = _lib.MAT_ELASTIC

    def _post_init(self) -> None:
        if self.model not in ("corotation", "neohooken"):
            raise GenesisException("model must be 'corotation' or 'neohooken'")

    def _flags(self) -> int:
        return _lib.MATF_NEOHOOKEAN if self.model == "neohooken" else 0


class Liquid(_MPMBase):
    """liquid.py:11-49: mu = 0 unless viscous."""

    _fields = ("viscous",)
    viscous = False
    _type = _lib.MAT_LIQUID

    def _post_init(self) -> None:
        if not self.viscous:
            self.mu = 0.0


class Sand(_MPMBase):
    """sand.py:11-45: Drucker-Prager, friction angle in degrees, default Jp 0."""

    _fields = ("friction_angle",)
    sampler = "random"
    friction_angle = 45.0
    _type = _lib.MAT_SAND
    _default_Jp = 0.0

    def _post_init(self) -> None:
        if not (self.friction_angle > 0):
            raise GenesisException("friction_angle must be positive")
        sin_phi = math.sin(math.radians(self.friction_angle))
        self.alpha = math.sqrt(2 / 3) * 2 * sin_phi / (3 - sin_phi)


class ElastoPlastic(_MPMBase):
    """elasto_plastic.py:10-71."""

    _fields = ("yield_lower", "yield_higher", "use_von_mises", "von_mises_yield_stress")
    yield_lower = 2.5e-2
    yield_higher = 4.5e-3
    use_von_mises = True
    von_mises_yield_stress = 10000.0
    _type = _lib.MAT_ELASTOPLASTIC

    def _flags(self) -> int:
        return _lib.MATF_VON_MISES if self.use_von_mises else 0


class Snow(ElastoPlastic):
    """snow.py:12-74: ElastoPlastic clamp with hardening; von Mises not supported."""

    sampler = "random"
    use_von_mises = False
    _type = _lib.MAT_SNOW

    def __init__(self, **kw):
        if kw.get("use_von_mises", False):
            raise GenesisException("Snow does not support use_von_mises=True.")
        kw["use_von_mises"] = False
        super().__init__(**kw)

    def _flags(self) -> int:
        return 0


class Muscle(Elastic):
    """muscle.py:9-53: Elastic (default neohooken, E 1e6) plus actuation stress."""

    _fields = ("n_groups",)
    E = 1e6
    model = "neohooken"
    n_groups = 1
    _type = _lib.MAT_MUSCLE

    def _post_init(self) -> None:
        super()._post_init()
        self.stiffness = self.E


class MPM:
    """Namespace matching gs.materials.MPM."""

    Elastic = Elastic
    Liquid = Liquid
    Sand = Sand
    Snow = Snow
    ElastoPlastic = ElastoPlastic
    Muscle = Muscle


class Tool:
    """genesis/engine/materials/tool.py:13-32: the material of a tool entity (a kinematic mesh
    that pushes MPM particles through its SDF in the grid op)."""

    _fields = ("friction", "coup_softness", "collision", "sdf_res")
    friction = 0.0
    coup_softness = 0.01
    collision = True
    sdf_res = 128

    def __init__(self, **kw):
        unknown = set(kw) - set(self._fields)
        if unknown:
            raise GenesisException(f"Unrecognized attribute(s) for Tool: {sorted(unknown)}")
        for f in self._fields:
            setattr(self, f, kw.get(f, getattr(type(self), f)))
        if not (self.friction >= 0) or not (self.coup_softness >= 0):
            raise GenesisException("Tool friction and coup_softness must be non-negative.")
        if not isinstance(self.collision, bool):
            raise GenesisException("Tool collision must be a bool.")
        if int(self.sdf_res) != self.sdf_res or self.sdf_res < 2:
            raise GenesisException("Tool sdf_res must be an integer >= 2.")
        self.sdf_res = int(self.sdf_res)
        self.idx = None

    def __eq__(self, other) -> bool:
        return type(self) is type(other) and all(getattr(self, f) == getattr(other, f) for f in self._fields)
