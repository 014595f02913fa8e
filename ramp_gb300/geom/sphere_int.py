from .sphere import GSphere
from .. import _abi


class GSphereInt(GSphere):
    """Interior of a sphere (mcramp/geom/sphere_int.py:9-81,
    sphere_int.cl:3-42): the positive-time exit is stored in both halves of
    the intersection.  Slots: gp[0]=radius."""
    kind = _abi.G_SPHERE_INT
