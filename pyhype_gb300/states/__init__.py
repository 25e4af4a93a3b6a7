"""Host-side state containers for initial conditions and boundary-condition values.

These mirror the parts of ``pyhype/states`` that user code touches before a solve:
``PrimitiveState(fluid, array=...)``, ``.to_type(ConservativeState)``, ``.data``,
``.make_non_dimensional()`` and the variable properties.  They are numpy-only and run
once at set-up; the time loop never touches them.  The conversions use the
reference's arithmetic order (``pyhype/states/converter/concrete_defs.py:85-141``,
``pyhype/states/primitive.py:93-103``, ``pyhype/states/conservative.py:85-124``) so an
initial condition built here is bit-identical to the reference's.
"""
from .base import State, RealizabilityException
from .primitive import PrimitiveState
from .conservative import ConservativeState

__all__ = ["State", "RealizabilityException", "PrimitiveState", "ConservativeState"]
