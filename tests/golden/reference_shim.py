"""Import the reference package (jesuspueblas/meshcfd) from a local checkout.

Test infrastructure only: used to generate the golden fixtures in this folder
and by CPU tests that compare against the live reference when a checkout is
present.  Numba is not installed here, so a stub ``numba.njit`` (identity
decorator) is registered first: the reference's compiled kernels then run as
plain Python with the same operation order.  PyQt5 is absent, so only the
non-GUI modules are imported.
"""

from __future__ import annotations

import os
import sys
import types
from pathlib import Path

# Where the reference package is looked for, first match wins: the directory
# named by MESHCFD_REFERENCE (a checkout with src/meshcfd, or a directory
# holding the meshcfd package), the offline install of the unmodified
# package under baseline/_ref of this repository (which travels with the
# repository to machines without a checkout), and the read-only checkout of
# the build container.
_REPO = Path(__file__).resolve().parents[2]
_CANDIDATES = [Path(p) for p in (os.environ.get("MESHCFD_REFERENCE"),) if p] + [
    _REPO / "baseline" / "_ref", Path("/root/reference")]


def _package_root():
    """The directory that holds the ``meshcfd`` package, or None."""
    for base in _CANDIDATES:
        for root in (base / "src", base):
            if (root / "meshcfd" / "core" / "solver.py").exists():
                return root
    return None


REFERENCE = _package_root()


def available() -> bool:
    return REFERENCE is not None


def import_reference():
    """Return the reference's ``meshcfd.core`` modules as a namespace."""
    if not available():
        raise ImportError("reference package not found (set MESHCFD_REFERENCE)")
    if "numba" not in sys.modules:
        stub = types.ModuleType("numba")
        stub.njit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
        sys.modules["numba"] = stub
    for p in (str(REFERENCE),):
        if p not in sys.path:
            sys.path.insert(0, p)
    from meshcfd.core import _kernels, euler, model, solver  # noqa: E402

    return types.SimpleNamespace(solver=solver, euler=euler, model=model, kernels=_kernels)


def import_reference_mesh_io():
    """Return the reference's ``meshcfd.io.mesh_io`` module."""
    import_reference()
    from meshcfd.io import mesh_io  # noqa: E402

    return mesh_io


def reference_case(case, ref):
    """Rebuild one of our cases with the reference's own dataclasses."""
    from meshcfd_gb300.meshes import to_reference_mesh

    m = ref.model
    mesh = to_reference_mesh(case.mesh, m.FiniteVolumeMesh)
    mesh.patches = tuple(m.MeshPatch(p.id, p.name, tuple(int(f) for f in p.face_ids)) for p in case.mesh.patches)
    rcase = m.Case(name=case.name, mesh=mesh)
    rcase.boundary_conditions = [
        m.BoundaryCondition(c.patch_id, c.patch_name, c.kind, dict(c.values), c.thermal_condition,
                            c.mechanical_condition)
        for c in case.boundary_conditions
    ]
    rcase.periodic_pairs = [m.PeriodicBoundaryPair(p.patch_a_id, p.patch_b_id, p.axis, p.pitch)
                            for p in case.periodic_pairs]
    for key, value in vars(case.numerics).items():
        setattr(rcase.numerics, key, value)
    return rcase
