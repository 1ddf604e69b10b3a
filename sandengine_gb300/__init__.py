"""sandengine_gb300: sandengine's Margolus grid update on GB300 (sm_103a).

The rule language (``lang``) compiles YAML rule sets to CUDA through the C++ front end of
libsandengine_gb300; ``Simulation`` advances one world on the GPU.  Both mirror the
reference's API (sandengine-lang, sandengine-core).
"""
from ._lib import ParseError, SandengineError  # noqa: F401
from .lang import Ruleset, create_glsl_from_parser, parse_path, parse_string  # noqa: F401
from .simulation import (MODSHAPE_CIRCLE, MODSHAPE_SQUARE, Params, SimModification,  # noqa: F401
                         Simulation, grid_digest)

__all__ = ["ParseError", "SandengineError", "Ruleset", "parse_string", "parse_path",
           "create_glsl_from_parser", "Simulation", "SimModification", "Params", "MODSHAPE_CIRCLE",
           "MODSHAPE_SQUARE", "grid_digest"]
