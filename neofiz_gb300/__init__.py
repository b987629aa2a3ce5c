"""neofiz_gb300: the Neofiz explicit central-difference timestep on GB300 (sm_103a).

The product is libneofiz_gpu.so (C ABI in include/neofiz.h); this package is its host-side
mirror of the reference's Java API (ExplicitSolver, RigidWall, Contact), the mesh and material
inputs that feed it, and the in-tree build.
"""
from .materials import Formulation, Integration, Kinematics, JohnsonCook, Material, Materials
from .mesh import QuadMesh, Outline
from .solver import ExplicitSolver, RigidWall, Contact, material_point_update

__all__ = ["Formulation", "Integration", "Kinematics", "JohnsonCook", "Material", "Materials",
           "QuadMesh", "Outline", "ExplicitSolver", "RigidWall", "Contact",
           "material_point_update"]
