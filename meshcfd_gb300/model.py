"""Case description objects for the GB300 residual/step path.

These mirror the reference data model (``src/meshcfd/core/model.py``) field for
field, so that a case built for the reference solver and a case built here carry
the same meaning.  Mesh arrays may be NumPy arrays instead of tuples, which keeps
multi-million-cell meshes cheap to build.

Reference interfaces mirrored:
  * ``FiniteVolumeMesh``      model.py:60-74
  * ``MeshPatch``             model.py:37-41
  * ``BoundaryCurve``         model.py:44-49
  * ``RefinementRecord``      model.py:52-57
  * ``BoundaryCondition``     model.py:77-84
  * ``PeriodicBoundaryPair``  model.py:87-92
  * ``NumericalSettings``     model.py:95-129
  * ``InitialState``          model.py:132-139
  * ``Case``                  model.py:158-182
  * scheme name tuples        model.py:9-34
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

BOUNDARY_TYPES = (
    "Wall",
    "Velocity Inlet",
    "Pressure Inlet",
    "Pressure Outlet",
    "Mass Flow Inlet",
    "Mass Flow Outlet",
    "Symmetry",
    "Far Field",
    "Periodic",
)
RECONSTRUCTION_SCHEMES = ("First order", "MUSCL linear", "MUSCL parabolic")
LIMITER_SCHEMES = ("Barth-Jespersen", "Venkatakrishnan", "Minmod", "Van Leer")
FLUX_SCHEMES = ("HLLC", "Roe", "Rusanov")
TIME_INTEGRATION_SCHEMES = (
    "Explicit Euler",
    "Explicit RK2",
    "Explicit RK3",
    "Explicit RK4",
    "Implicit Euler",
)
TIME_STEP_MODES = ("Global adaptive", "Global fixed", "Local (steady)")

# Kernel codes.  The limiter codes are the ones the reference hands to its
# compiled limiter (solver.py:2303-2308); the flux codes follow the order of
# the dispatch in euler.py:67-72.
FLUX_CODES = {"Rusanov": 0, "HLLC": 1, "Roe": 2}
RECONSTRUCTION_CODES = {"First order": 0, "MUSCL linear": 1, "MUSCL parabolic": 2}
LIMITER_CODES = {"Barth-Jespersen": 0, "Minmod": 1, "Van Leer": 2, "Venkatakrishnan": 3}
# Extension with no counterpart in the reference: Venkatakrishnan's limiter in
# its published form with the smoothing constant K (limiter code 4), chosen
# with ``limiter = "Venkatakrishnan K"``; K is the settings attribute
# ``venkatakrishnan_k`` (default VENKATAKRISHNAN_K_DEFAULT).
EXTENSION_LIMITER_CODES = {"Venkatakrishnan K": 4}
VENKATAKRISHNAN_K_DEFAULT = 5.0


@dataclass
class MeshPatch:
    id: int
    name: str
    face_ids: Any


@dataclass(frozen=True)
class BoundaryCurve:
    geometry: dict
    start_parameter: float
    end_parameter: float
    patch_id: int


@dataclass(frozen=True)
class RefinementRecord:
    parent_id: str
    child_ids: tuple
    vertices: tuple
    level: int


@dataclass
class FiniteVolumeMesh:
    """Polygonal 2D mesh.  Arrays: points (N,2) float, faces (F,2) int,
    face_owners/face_neighbours/face_patch_ids (F,) int.  ``cells`` is a
    sequence of vertex-id sequences, or a (C,k) int array for single-shape
    meshes, or a :class:`CellArray` for mixed shapes."""

    points: Any
    cells: Any
    faces: Any
    face_owners: Any
    face_neighbours: Any
    face_patch_ids: Any
    patches: tuple
    cell_face_ids: Any = ()
    cell_face_signs: Any = ()
    cell_ids: tuple = ()
    cell_levels: tuple = ()
    refinement_records: tuple = ()
    face_curves: tuple = ()


@dataclass
class BoundaryCondition:
    patch_id: int
    patch_name: str
    kind: str = "Wall"
    values: dict = field(default_factory=dict)
    thermal_condition: str = "Temperature"
    mechanical_condition: str = "No-slip"


@dataclass(frozen=True)
class PeriodicBoundaryPair:
    patch_a_id: int
    patch_b_id: int
    axis: str
    pitch: float


@dataclass
class NumericalSettings:
    reconstruction: str = "MUSCL linear"
    limiter: str = "Barth-Jespersen"
    flux: str = "HLLC"
    time_integration: str = "Explicit RK2"
    time_step_mode: str = "Global adaptive"
    cfl: float = 0.5
    fixed_time_step: float = 0.001
    gmres_tolerance: float = 1e-6
    gmres_max_iterations: int = 300
    gmres_krylov_dimension: int = 30
    implicit_preconditioner: str = "LU-SGS"
    max_iterations: int = 1000
    end_time: float = 1.0
    residual_tolerance: float = 1e-6
    convergence_history_interval: int = 10
    gamma: float = 1.4
    gas_constant: float = 287.05
    viscosity_model: str = "Inviscid"
    dynamic_viscosity: float = 1.8e-5
    sutherland_reference_viscosity: float = 1.716e-5
    sutherland_reference_temperature: float = 273.15
    sutherland_temperature: float = 110.4
    prandtl_number: float = 0.72
    acceleration_x: float = 0.0
    acceleration_y: float = 0.0
    adaptive_mesh: bool = False
    adaptation_interval: int = 20
    adaptation_max_level: int = 3
    adaptation_refine_threshold: float = 0.25
    adaptation_variable: str = "Density"
    turbulence_model: str = "None"
    turbulence_wall_treatment: str = "Wall-resolved"
    turbulence_omega_formulation: str = "Standard SST"


@dataclass
class InitialState:
    density: float = 1.225
    velocity_x: float = 0.0
    velocity_y: float = 0.0
    pressure: float = 101325.0
    turbulence_k: float = 1e-6
    turbulence_omega: float = 1.0


@dataclass
class Case:
    name: str = "Untitled"
    mesh: FiniteVolumeMesh | None = None
    boundary_conditions: list = field(default_factory=list)
    numerics: NumericalSettings = field(default_factory=NumericalSettings)
    periodic_pairs: list = field(default_factory=list)

    def __post_init__(self) -> None:
        if self.mesh is not None and not self.boundary_conditions:
            self.boundary_conditions = [
                BoundaryCondition(patch.id, patch.name) for patch in self.mesh.patches
            ]

    def condition(self, name: str) -> BoundaryCondition:
        for condition in self.boundary_conditions:
            if condition.patch_name == name:
                return condition
        raise KeyError(name)
