"""Initial conditions run on the host against block proxies (``block.mesh.x/y``,
``block.state``, ``block.config``), as ``pyhype/initial_conditions/base.py:28-31``."""
from __future__ import annotations

from abc import ABC, abstractmethod


class InitialCondition(ABC):
    @abstractmethod
    def apply_to_block(self, block):
        raise NotImplementedError("Abstract Initial Condition")
