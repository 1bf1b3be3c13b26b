"""The reference's exception types, for the Python host side.

Julia's ``error(msg)`` raises an ``ErrorException`` and a size check a
``DimensionMismatch``; callers of WesterveltEDG.jl match on those types and on
the messages. ``ArgumentErrorException`` is the ``ErrorException`` of a bad
argument (the checks of ``precompute`` and of the flux and boundary helpers,
src/solver.jl:16-66, 437-440, 744-747); it is also a ``ValueError`` so that
Python callers can catch it as one.
"""


class ErrorException(RuntimeError):
    """The reference's ErrorException (its own error messages, e.g. src/rhs.jl:114-115, 845, 916)."""


class DimensionMismatch(ValueError):
    """The reference's DimensionMismatch (src/rhs.jl:500-503)."""


class ArgumentErrorException(ErrorException, ValueError):
    """An ErrorException raised for a bad argument (src/solver.jl:20, 56-66, 191, 438-440, 746)."""
