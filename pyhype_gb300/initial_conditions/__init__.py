from .base import InitialCondition
from .explosion import ExplosionInitialCondition, SupersonicFloodInitialCondition

__all__ = ["InitialCondition", "ExplosionInitialCondition", "SupersonicFloodInitialCondition"]
