"""Moderator plugins (mcramp/moderator/*)."""
from .flat_mod import MFlat
from .cont_mod import MCont
from .isis_mod import MISIS
