"""Geometry build on the GPU.

``build_geometry(mesh, case, host=DeviceGeometryBuilder())`` runs the
numeric loops of the reference's ``_build_geometry`` (solver.py:1654-2105)
in the library's kernels (``csrc/mcfd_geometry.cu``): cell centroids and
areas, face centres, normals and lengths, the least-squares gradient
offsets, weights, moment sums and coefficients, and the limiter-entry
offsets.  The topology (the index lists, periodic matching, boundary
classification) stays on the host, as it does in the reference.  The
kernels keep the host build's operation order, so the resulting
``Geometry`` is the host build's bit for bit.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .errors import SolverError


_NONE = np.iinfo(np.int64).max  # no bad cell / face (the kernels keep the smallest bad index)


def _t(a, dev, dtype):
    """A device copy of ``a``; keep the tensor referenced until the kernel that
    reads it has run (a temporary's memory returns to the caching allocator
    at once and may be handed to the next copy)."""
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)


class DeviceGeometryBuilder:
    """The ``host`` hooks of :func:`geometry.build_geometry`, run on a CUDA
    device; no CPU fallback (a missing device raises)."""

    def __init__(self, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("DeviceGeometryBuilder needs a CUDA device (no CPU fallback)")
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.lib = _lib.native()
        self._cells = None

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def cell_geometry(self, offsets, nodes, points):
        """Centroids and areas (mcfd_device_cell_geometry)."""
        dev = self.device
        n = len(offsets) - 1
        pts = _t(points, dev, torch.float64)
        centers = torch.empty(n, 2, dtype=torch.float64, device=dev)
        areas = torch.empty(n, dtype=torch.float64, device=dev)
        bad = torch.full((1,), _NONE, dtype=torch.int64, device=dev)
        off, nd = _t(offsets, dev, torch.int64), _t(nodes, dev, torch.int64)  # alive until the kernel has run
        self.lib.check(self.lib.mcfd_device_cell_geometry(
            n, off.data_ptr(), nd.data_ptr(), pts.data_ptr(), centers.data_ptr(), areas.data_ptr(), bad.data_ptr(),
            self._stream()), "mcfd_device_cell_geometry")
        first = int(bad.item())
        if first != _NONE:
            raise SolverError(f"Cell {first} has zero or invalid area.")
        self._cells = (pts, centers)
        return centers.cpu().numpy(), areas.cpu().numpy()

    def face_geometry(self, faces, points, centers, owners):
        """Face centres, outward unit normals and lengths
        (mcfd_device_face_geometry)."""
        dev = self.device
        if self._cells is not None:
            pts, cen = self._cells
        else:
            pts, cen = _t(points, dev, torch.float64), _t(centers, dev, torch.float64)
        fn = _t(np.asarray(faces).reshape(-1, 2), dev, torch.int64)
        n = fn.shape[0]
        fc = torch.empty(n, 2, dtype=torch.float64, device=dev)
        nrm = torch.empty(n, 2, dtype=torch.float64, device=dev)
        ln = torch.empty(n, dtype=torch.float64, device=dev)
        bad = torch.full((1,), _NONE, dtype=torch.int64, device=dev)
        own = _t(owners, dev, torch.int64)
        self.lib.check(self.lib.mcfd_device_face_geometry(
            n, fn.data_ptr(), pts.data_ptr(), cen.data_ptr(), own.data_ptr(), fc.data_ptr(), nrm.data_ptr(),
            ln.data_ptr(), bad.data_ptr(), self._stream()), "mcfd_device_face_geometry")
        first = int(bad.item())
        if first != _NONE:
            raise SolverError(f"Face {first} has zero or invalid length.")
        return fc.cpu().numpy(), nrm.cpu().numpy(), ln.cpu().numpy()

    def gradient_and_limiter_offsets(self, n_cells, src, nbr, n_interior_entries, shifts, centers, face_centers,
                                     slot_faces, slot_cells):
        """(gdx, gdy, cx, cy, limiter dx, limiter dy) of the entry lists."""
        dev = self.device
        n = len(src)
        s_t, n_t = _t(src, dev, torch.int64), _t(nbr, dev, torch.int64)
        cen = _t(centers, dev, torch.float64)
        fc = _t(face_centers, dev, torch.float64)
        sh = _t(np.asarray(shifts, dtype=float).reshape(-1, 2), dev, torch.float64)
        order = np.argsort(src, kind="stable")
        ptr = np.concatenate(([0], np.cumsum(np.bincount(src, minlength=n_cells)))).astype(np.int64)
        o_t, p_t = _t(order, dev, torch.int64), _t(ptr, dev, torch.int64)
        out = torch.empty(4, max(n, 1), dtype=torch.float64, device=dev)
        scratch = torch.empty(2 * n + 3 * n_cells, dtype=torch.float64, device=dev)
        self.lib.check(self.lib.mcfd_device_gradient_coefficients(
            n_cells, n, int(n_interior_entries), s_t.data_ptr(), n_t.data_ptr(), cen.data_ptr(),
            sh.data_ptr() if sh.numel() else None, p_t.data_ptr(), o_t.data_ptr(), out[0].data_ptr(),
            out[1].data_ptr(), out[2].data_ptr(), out[3].data_ptr(), scratch.data_ptr(), self._stream()),
            "mcfd_device_gradient_coefficients")
        ns = len(slot_faces)
        lim = torch.empty(2, max(ns, 1), dtype=torch.float64, device=dev)
        sf, sc = _t(slot_faces, dev, torch.int64), _t(slot_cells, dev, torch.int64)
        self.lib.check(self.lib.mcfd_device_limiter_offsets(
            ns, sf.data_ptr(), sc.data_ptr(), fc.data_ptr(), cen.data_ptr(), lim[0].data_ptr(), lim[1].data_ptr(),
            self._stream()), "mcfd_device_limiter_offsets")
        g = out[:, :n].cpu().numpy()
        lm = lim[:, :ns].cpu().numpy()
        return g[0].copy(), g[1].copy(), g[2].copy(), g[3].copy(), lm[0].copy(), lm[1].copy()

    def parabolic_stencil(self, *args):
        return self.lib.parabolic_stencil(*args)
