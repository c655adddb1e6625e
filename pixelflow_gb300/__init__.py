"""pixelflow_gb300: GB300-native immersed-boundary step of PixelFlow.

The compute path is libpixelflow_gb300.so (hand-written sm_103a kernels
behind the C ABI of include/pixelflow_gpu.h); this package is its host-side
mirror: reference-compatible inputs (config), synthetic geometries, and the
`Case` object whose methods carry the reference's routine names.
"""
from .config import Settings, read_porosity_csv, read_settings, write_porosity_csv, write_settings  # noqa: F401

__all__ = ["Settings", "read_settings", "write_settings", "read_porosity_csv", "write_porosity_csv",
           "Case", "build"]


def build(force: bool = False, verbose: bool = False) -> str:
    from . import buildlib as _b
    return _b.build(force=force, verbose=verbose)


def __getattr__(name):
    if name == "Case":
        from .solver import Case
        return Case
    raise AttributeError(name)
