from .base import PrimitiveDirichletBC  # noqa: F401  (reference module path)
