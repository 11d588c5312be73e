"""GB300 (sm_103a) implementation of the WumingPIC2D time step.

    layout      reference-layout host arrays (Dims)
    api         the common/ module procedures (particle__solv, field__fdtd_i, ...)
    sim         resident simulation (Simulation): state kept on the GPU across steps
    weibel      seeded two-beam Weibel initial condition
    build       compiles csrc/*.cu into _lib/libwmpic2d.so
"""
from .layout import Dims, bits_to_pid, pid_to_bits  # noqa: F401

__all__ = ["Dims", "pid_to_bits", "bits_to_pid"]
