"""Geometry plugins (mcramp/geom/*)."""
from .gprim import GPrim
from .plane import GPlane
from .cylinder_ext import GCylinderExt
from .banana import GBanana
from .sphere import GSphere
from .sphere_int import GSphereInt
from .box import GBox
from .arm import GArm
from .mesh import GMesh, read_stl, write_stl
