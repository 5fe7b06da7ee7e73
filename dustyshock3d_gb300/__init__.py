"""GB300-native (sm_103a) drop-in for DustyShock3D's per-step dusty-gas SPH + IDIC path."""
from .params import Mode, Params, parse_init_txt, read_init_txt, write_init_txt  # noqa: F401
from .species import Species  # noqa: F401
from . import ic  # noqa: F401
