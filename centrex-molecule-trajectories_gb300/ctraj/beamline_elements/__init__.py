from .apertures import *  # noqa: F401,F403
from .electrostatic_lens import *  # noqa: F401,F403
from .meshes import *  # noqa: F401,F403
