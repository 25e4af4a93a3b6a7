from .base import MeshGenerator, QuadMeshGenerator
from .quad_mesh import BlockGeometry, QuadMesh, build_block_geometry
from .rectangular import RectagularMeshGenerator, RectangularMeshGenerator

__all__ = [
    "MeshGenerator", "QuadMeshGenerator", "BlockGeometry", "QuadMesh", "build_block_geometry",
    "RectagularMeshGenerator", "RectangularMeshGenerator",
]
