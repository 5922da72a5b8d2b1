"""chimeracl_gb300: the quasi-cylindrical PSATD particle-in-cell step of
chimeraCL, rebuilt for the GB300 (sm_103a) on hand-written CUDA kernels.

Drop-in for the reference's Python API: ``Grid``, ``Particles``, ``Solver``,
``Transformer``, ``Frame``, ``add_gausian_pulse``, ``PIC_loop`` and the
``Args``/``DataDev`` containers, with ``torch.Tensor`` device arrays and the
methods layer calling ``libchimeracl_gb300.so`` through its C ABI."""
__version__ = "0.1.0"

from .methods.generic_methods_cu import Communicator  # noqa: F401,E402


def __getattr__(name):
    # lazy imports keep `import chimeracl_gb300` light (no CUDA needed)
    if name == "Grid":
        from .grid import Grid
        return Grid
    if name == "Particles":
        from .particles import Particles
        return Particles
    if name == "Solver":
        from .solver import Solver
        return Solver
    if name == "Frame":
        from .frame import Frame
        return Frame
    if name == "PIC_loop":
        from .pic_loop import PIC_loop
        return PIC_loop
    if name == "PIC_batch":
        from .batch import PIC_batch
        return PIC_batch
    if name == "add_gausian_pulse":
        from .laser import add_gausian_pulse
        return add_gausian_pulse
    raise AttributeError(name)
