"""The methods layer: mixins that the wrapper classes inherit, one per
reference module of chimeraCL/methods/ (``*_methods_cl.py`` there,
``*_methods_cu.py`` here), with the same method names and arguments."""
from .generic_methods_cu import Communicator, GenericMethodsCU  # noqa: F401
from .grid_methods_cu import GridMethodsCU  # noqa: F401
from .particles_methods_cu import ParticleMethodsCU  # noqa: F401
from .solver_methods_cu import SolverMethodsCU  # noqa: F401
from .transformer_methods_cu import TransformerMethodsCU  # noqa: F401
