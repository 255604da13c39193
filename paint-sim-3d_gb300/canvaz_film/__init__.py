"""canvaz_film — GB300 (sm_103a) thin-film step of Canvaz behind a C ABI.

The product is the CUDA library built from ../csrc (libcanvaz_film.so,
include/canvaz_film.h).  This package is its Python host side: ctypes
bindings (capi), the Film mirror of the reference's `impl Film` (film),
seeded synthetic canvases (synth), batching (batch) and serving (serve).
"""
from . import capi  # noqa: F401
from .capi import Settings, Params  # noqa: F401
