"""The reference's ``qaravan.core`` surface used by the simulators: circuits,
gates (fixed and parametrised), noise models, Pauli helpers, the TFI
Hamiltonian and ``RunContext``. ``from qaravan_gb300.core import *`` replaces
``from qaravan.core import *`` for circuit construction (host objects; the
simulators in ``qaravan_gb300.tensorQ`` also accept the reference's own)."""
from .circuits import *  # noqa: F401,F403
from .environments import RunContext  # noqa: F401
from .gates import *  # noqa: F401,F403
from .hamiltonians import *  # noqa: F401,F403
from .noise import *  # noqa: F401,F403
from .paulis import *  # noqa: F401,F403
from .skeletons import *  # noqa: F401,F403
from .applications.compilation import string_to_sv  # noqa: F401  (core/utils.py:46-50)
from .measure import pretty_print_dm, pretty_print_sv  # noqa: F401  (core/utils.py:52-89)
