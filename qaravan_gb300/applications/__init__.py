"""Applications of the reference (``applications/``) on the GPU."""
from .compilation import *  # noqa: F401,F403
from .trotter import *  # noqa: F401,F403
