"""GB300 (sm_103a) backend for GeneralizedGrossPitaevskii.jl's StrangSplitting solver.

The compute path is libgpe.so (C ABI in include/gpe.h, CUDA sources in csrc/); this
package is the host-side mirror of the reference's Julia surface:

    prob = GrossPitaevskiiProblem(u0, lengths; dispersion, potential, nonlinearity,
                                  pump, position_noise_func, noise_prototype, param)
    ts, result = solve(prob, StrangSplitting(), tspan, dt=..., nsaves=...)

(src/problem.jl:97-123, src/fixed_time_stepping.jl:56-81).
"""
from ._lib import GPEError, load as load_library
from .problem import (GrossPitaevskiiProblem, SeparablePump, direct_grid, reciprocal_grid)
from .strang import (StrangSplitting, StrangSplittingIterator, init, pump_sample_times,
                     resolve_fixed_timestepping, solve, solve_, step)

__all__ = [
    "GrossPitaevskiiProblem", "SeparablePump", "StrangSplitting", "StrangSplittingIterator", "init",
    "solve", "solve_", "step", "direct_grid", "reciprocal_grid", "resolve_fixed_timestepping", "pump_sample_times",
    "GPEError", "load_library", "build",
]


def build(force: bool = False, verbose: bool = False):
    """Compile libgpe.so for sm_103a (see build.py)."""
    from .build import build as _build
    return _build(force=force, verbose=verbose)
