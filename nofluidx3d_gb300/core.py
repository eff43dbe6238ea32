"""Thin Python handle over the C ABI: one `CellSim` is one nfx_sim (one cell on one GPU).

Arrays cross the boundary in the reference's layouts (points/velocities SoA float64 3*Np,
tetras SoA uint32 4*Nt); the convenience methods here accept and return (N, 3) / (Nt, 4)
arrays and convert. Every call goes to libnfx; failures raise NfxError.
"""

from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import (CONTACT_PLANE, CONTACT_SPHERE, CONTACT_SUBSTRATE, FIELD_PLASTIC_STRAIN, FIELD_PRESSURE,
                   FIELD_VON_MISES, MODEL_MR, MODEL_SVK, MODEL_SVKK, MODEL_VP, NfxError, check)

__all__ = ["CellSim", "Batch", "NfxError", "MODEL_MR", "MODEL_SVK", "MODEL_SVKK", "MODEL_VP", "CONTACT_SUBSTRATE",
           "CONTACT_PLANE", "CONTACT_SPHERE", "FIELD_VON_MISES", "FIELD_PRESSURE", "FIELD_PLASTIC_STRAIN",
           "to_soa", "from_soa"]


def to_soa(a: np.ndarray, dtype=np.float64) -> np.ndarray:
    """(N, k) -> contiguous k*N SoA vector (the reference's order='F' reshape, Simulation.py:82-87)."""
    a = np.asarray(a)
    return np.ascontiguousarray(a.T.reshape(-1), dtype=dtype)


def from_soa(v: np.ndarray, k: int) -> np.ndarray:
    """k*N SoA vector -> (N, k)."""
    return np.asarray(v).reshape(k, -1).T


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class PinnedArray:
    """A float64 numpy array in page-locked host memory (nfx_host_alloc), for output snapshots
    whose copies overlap the steps; the memory is freed with the object."""

    def __init__(self, n: int):
        self._L = _lib.load()
        p = C.c_void_p()
        check(self._L.nfx_host_alloc(8 * max(int(n), 1), C.byref(p)))
        self._p = p
        self.array = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), shape=(max(int(n), 1),))[:int(n)]

    def __del__(self):
        try:
            if getattr(self, "_p", None) is not None and self._p.value:
                self.array = None
                self._L.nfx_host_free(self._p)
                self._p = None
        except Exception:
            pass


class CellSim:
    """One cell simulation on a CUDA device (see include/nfx.h for the semantics of each call)."""

    def __init__(self, device: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        check(self._L.nfx_create(int(device), C.byref(h)))
        self._h = h
        self.device = device
        self.np = 0
        self.nt = 0
        self.n_contacts = 0

    # ------------------------------------------------------------------ lifecycle
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.nfx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ set-up
    def set_mesh(self, points: np.ndarray, tets: np.ndarray) -> None:
        pts = to_soa(points, np.float64)
        tt = to_soa(tets, np.uint32)
        np_, nt = int(np.asarray(points).shape[0]), int(np.asarray(tets).shape[0])
        check(self._L.nfx_set_mesh(self._h, np_, nt, _ptr(pts), _ptr(tt)))
        self.np, self.nt = np_, nt

    def set_mesh_soa(self, np_: int, nt: int, points_soa: np.ndarray, tets_soa: np.ndarray) -> None:
        pts = np.ascontiguousarray(points_soa, np.float64)
        tt = np.ascontiguousarray(tets_soa, np.uint32)
        check(self._L.nfx_set_mesh(self._h, int(np_), int(nt), _ptr(pts), _ptr(tt)))
        self.np, self.nt = int(np_), int(nt)

    def set_tetra(self, model: int, youngs: float, poisson: float, mr_ratio: float = 1.0) -> None:
        check(self._L.nfx_set_tetra(self._h, int(model), float(youngs), float(poisson), float(mr_ratio)))

    def set_viscoplastic(self, par: Sequence[float]) -> None:
        p = np.ascontiguousarray(par, np.float64)
        if p.size != 8:
            raise ValueError("8 viscoplastic parameters expected")
        check(self._L.nfx_set_viscoplastic(self._h, _ptr(p)))

    def add_contact(self, kind: int, k: float, radius: float = 0.0, p0: float = 0.0, v: float = 0.0,
                    tmove: float = float("inf")) -> int:
        cid = C.c_int(-1)
        check(self._L.nfx_add_contact(self._h, int(kind), float(k), float(radius), float(p0), float(v),
                                      float(tmove), C.byref(cid)))
        self.n_contacts += 1
        return cid.value

    def set_contact_table(self, cid: int, t0: int, positions: np.ndarray | None) -> None:
        if positions is None or len(positions) == 0:
            check(self._L.nfx_set_contact_table(self._h, int(cid), int(t0), 0, None))
            return
        p = np.ascontiguousarray(positions, np.float64)
        check(self._L.nfx_set_contact_table(self._h, int(cid), int(t0), int(p.size), _ptr(p)))

    def set_integrator(self, xi: float, fix_top_bottom: bool = False) -> None:
        check(self._L.nfx_set_integrator(self._h, float(xi), int(bool(fix_top_bottom))))

    def set_integrator_lumped(self, xi: float, density: float = 1.0) -> None:
        """Lumped-mass velocity Verlet (velocityVerlet2.cl)."""
        check(self._L.nfx_set_integrator_lumped(self._h, float(xi), float(density)))

    def set_record(self, contact: int, every: int, max_rows: int) -> None:
        check(self._L.nfx_set_record(self._h, int(contact), int(every), int(max_rows)))

    # ------------------------------------------------------------------ stepping
    def step(self, n: int = 1) -> None:
        check(self._L.nfx_step(self._h, int(n)))

    def record_now(self) -> None:
        check(self._L.nfx_record_now(self._h))

    def sync(self) -> None:
        check(self._L.nfx_sync(self._h))

    def snapshot(self, points_out: np.ndarray, rows_out: np.ndarray | None = None) -> int:
        """Start an asynchronous copy of the node positions (SoA, 3*np doubles) and the recorded
        force rows (rows_out: [max_rows, 3] doubles) taken after the steps enqueued so far; later
        steps may be enqueued at once. Read the buffers only after snapshot_wait(). Returns the
        number of rows recorded so far."""
        assert points_out.dtype == np.float64 and points_out.flags.c_contiguous and points_out.size == 3 * self.np
        rows = 0 if rows_out is None else rows_out.shape[0]
        if rows_out is not None:
            assert rows_out.dtype == np.float64 and rows_out.flags.c_contiguous and rows_out.shape[1:] == (3,)
        n = C.c_int64()
        check(self._L.nfx_snapshot(self._h, _ptr(points_out), None if rows_out is None else _ptr(rows_out), rows,
                                   C.byref(n)))
        return n.value

    def snapshot_wait(self) -> None:
        """Wait for the copies of the latest snapshot."""
        check(self._L.nfx_snapshot_wait(self._h))

    @property
    def time(self) -> int:
        t = C.c_int64()
        check(self._L.nfx_get_time(self._h, C.byref(t)))
        return t.value

    # ------------------------------------------------------------------ state access
    def _get3(self, fn) -> np.ndarray:
        out = np.empty(3 * self.np, np.float64)
        check(fn(self._h, _ptr(out)))
        return out

    def points_soa(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(3 * self.np, np.float64)
        check(self._L.nfx_get_points(self._h, _ptr(out)))
        return out

    def points(self) -> np.ndarray:
        return from_soa(self.points_soa(), 3)

    def set_points(self, pts: np.ndarray) -> None:
        a = to_soa(pts) if np.asarray(pts).ndim == 2 else np.ascontiguousarray(pts, np.float64)
        check(self._L.nfx_set_points(self._h, _ptr(a)))

    def velocities(self) -> np.ndarray:
        return from_soa(self._get3(self._L.nfx_get_velocities), 3)

    def set_velocities(self, v: np.ndarray) -> None:
        a = to_soa(v) if np.asarray(v).ndim == 2 else np.ascontiguousarray(v, np.float64)
        check(self._L.nfx_set_velocities(self._h, _ptr(a)))

    def force_old(self) -> np.ndarray:
        return from_soa(self._get3(self._L.nfx_get_force_old), 3)

    def set_force_old(self, f: np.ndarray) -> None:
        a = to_soa(f) if np.asarray(f).ndim == 2 else np.ascontiguousarray(f, np.float64)
        check(self._L.nfx_set_force_old(self._h, _ptr(a)))

    def tet_field(self, which: int) -> np.ndarray:
        out = np.empty(self.nt, np.float64)
        check(self._L.nfx_get_tet_field(self._h, int(which), _ptr(out)))
        return out

    def plastic_tensor_soa(self) -> np.ndarray:
        out = np.empty(9 * self.nt, np.float64)
        check(self._L.nfx_get_plastic_tensor(self._h, _ptr(out)))
        return out

    def set_plastic_tensor_soa(self, fp: np.ndarray) -> None:
        """Overwrite Fp (SoA 9*nt doubles, user tetra order); the plastic strain is kept."""
        a = np.ascontiguousarray(fp, np.float64)
        if a.size != 9 * self.nt:
            raise ValueError("9*nt values expected")
        check(self._L.nfx_set_plastic_tensor(self._h, _ptr(a)))

    def checkpoint(self) -> bytes:
        """The whole state (after the enqueued steps) as an opaque byte string for restore()."""
        n = C.c_int64()
        check(self._L.nfx_checkpoint_size(self._h, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        check(self._L.nfx_checkpoint_save(self._h, _ptr(buf), n.value))
        return buf.tobytes()

    def restore(self, data: bytes) -> None:
        """Restore a checkpoint() into a handle set up with the same mesh and material model."""
        buf = np.frombuffer(data, np.uint8)
        check(self._L.nfx_checkpoint_load(self._h, buf.ctypes.data, buf.size))

    def curve(self, max_rows: int = 1 << 20) -> np.ndarray:
        n = C.c_int64()
        check(self._L.nfx_get_curve(self._h, None, 0, C.byref(n)))
        rows = min(n.value, max_rows)
        out = np.zeros((max(rows, 1), 3), np.float64)
        check(self._L.nfx_get_curve(self._h, _ptr(out), rows, C.byref(n)))
        return out[:rows]

    def indenter_force(self, contact: int) -> float:
        out = C.c_double()
        check(self._L.nfx_indenter_force(self._h, int(contact), C.byref(out)))
        return out.value

    def status(self, clear: bool = False) -> int:
        f = C.c_uint32()
        check(self._L.nfx_status(self._h, C.byref(f), int(bool(clear))))
        return f.value

    def time_steps(self, n: int) -> float:
        """Run n steps; device milliseconds between CUDA events on the handle's stream."""
        ms = C.c_float()
        check(self._L.nfx_time_steps(self._h, int(n), C.byref(ms)))
        return ms.value

    def profile_steps(self, n: int) -> tuple[float, float]:
        """Run n steps launch by launch; summed device ms of (element passes, node passes)."""
        a, b = C.c_float(), C.c_float()
        check(self._L.nfx_profile_steps(self._h, int(n), C.byref(a), C.byref(b)))
        return a.value, b.value

    def profile_tet_pass(self, launches: int) -> float:
        """Average device ms of one element pass over `launches` back-to-back launches (its
        effects on the state are undone)."""
        ms = C.c_float()
        check(self._L.nfx_profile_tet_pass(self._h, int(launches), C.byref(ms)))
        return ms.value

    def mesh_info(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        check(self._L.nfx_mesh_info(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value


class Batch:
    """Many independent cells advanced together (nfx_batch_*, include/nfx.h)."""

    def __init__(self, device: int = 0, tile_tets: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        check(self._L.nfx_batch_create(int(device), int(tile_tets), C.byref(h)))
        self._h = h
        self.cells: list[tuple[int, int]] = []  # (np, nt) per cell

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.nfx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_cell(self, points: np.ndarray, tets: np.ndarray) -> int:
        pts = to_soa(points, np.float64)
        tt = to_soa(tets, np.uint32)
        cid = C.c_int(-1)
        np_, nt = int(np.asarray(points).shape[0]), int(np.asarray(tets).shape[0])
        check(self._L.nfx_batch_add_cell(self._h, np_, nt, _ptr(pts), _ptr(tt), C.byref(cid)))
        self.cells.append((np_, nt))
        return cid.value

    def add_cell_like(self, src: int) -> int:
        """A new cell with the same mesh as cell `src` (shared, not copied)."""
        cid = C.c_int(-1)
        check(self._L.nfx_batch_add_cell_like(self._h, int(src), C.byref(cid)))
        self.cells.append(self.cells[src])
        return cid.value

    def set_tetra(self, cell: int, model: int, youngs: float, poisson: float, mr_ratio: float = 1.0) -> None:
        check(self._L.nfx_batch_set_tetra(self._h, int(cell), int(model), float(youngs), float(poisson), float(mr_ratio)))

    def set_viscoplastic(self, cell: int, par: Sequence[float]) -> None:
        p = np.ascontiguousarray(par, np.float64)
        check(self._L.nfx_batch_set_viscoplastic(self._h, int(cell), _ptr(p)))

    def add_contact(self, cell: int, kind: int, k: float, radius: float = 0.0, p0: float = 0.0, v: float = 0.0,
                    tmove: float = float("inf")) -> int:
        cid = C.c_int(-1)
        check(self._L.nfx_batch_add_contact(self._h, int(cell), int(kind), float(k), float(radius), float(p0),
                                            float(v), float(tmove), C.byref(cid)))
        return cid.value

    def set_integrator(self, cell: int, xi: float, fix_top_bottom: bool = False) -> None:
        check(self._L.nfx_batch_set_integrator(self._h, int(cell), float(xi), int(bool(fix_top_bottom))))

    def set_integrator_lumped(self, cell: int, xi: float, density: float = 1.0) -> None:
        check(self._L.nfx_batch_set_integrator_lumped(self._h, int(cell), float(xi), float(density)))

    def set_record(self, contact: int, every: int, max_rows: int) -> None:
        check(self._L.nfx_batch_set_record(self._h, int(contact), int(every), int(max_rows)))

    def finalize(self) -> None:
        check(self._L.nfx_batch_finalize(self._h))

    def step(self, n: int) -> None:
        check(self._L.nfx_batch_step(self._h, int(n)))

    def time_steps(self, n: int) -> float:
        ms = C.c_float()
        check(self._L.nfx_batch_time_steps(self._h, int(n), C.byref(ms)))
        return ms.value

    def record_now(self) -> None:
        check(self._L.nfx_batch_record_now(self._h))

    def cell_status(self, clear: bool = False) -> np.ndarray:
        """Status bits of every cell (NFX_STATUS_*)."""
        out = np.zeros(len(self.cells), np.uint32)
        check(self._L.nfx_batch_cell_status(self._h, _ptr(out), int(bool(clear))))
        return out

    def indenter_force(self, contact: int) -> np.ndarray:
        """Current force on contact index `contact` of every cell (0 where a cell has fewer)."""
        out = np.zeros(len(self.cells), np.float64)
        check(self._L.nfx_batch_indenter_force(self._h, int(contact), _ptr(out)))
        return out

    def curve(self, cell: int) -> np.ndarray:
        n = C.c_int64()
        check(self._L.nfx_batch_get_curve(self._h, int(cell), None, 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), 3), np.float64)
        check(self._L.nfx_batch_get_curve(self._h, int(cell), _ptr(out), n.value, C.byref(n)))
        return out[:n.value]

    def points(self, cell: int) -> np.ndarray:
        out = np.empty(3 * self.cells[cell][0], np.float64)
        check(self._L.nfx_batch_get_points(self._h, int(cell), _ptr(out)))
        return from_soa(out, 3)

    def set_points(self, cell: int, pts: np.ndarray) -> None:
        """Overwrite the node positions of one cell ((np, 3) or SoA 3*np doubles)."""
        a = to_soa(pts) if np.asarray(pts).ndim == 2 else np.ascontiguousarray(pts, np.float64)
        if a.size != 3 * self.cells[cell][0]:
            raise ValueError("3*np positions expected")
        check(self._L.nfx_batch_set_points(self._h, int(cell), _ptr(a)))

    def status(self, clear: bool = False) -> int:
        f = C.c_uint32()
        check(self._L.nfx_batch_status(self._h, C.byref(f), int(bool(clear))))
        return f.value

    def info(self) -> dict:
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int()
        check(self._L.nfx_batch_info(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        tiles = (C.c_int * 9)()
        ms = (C.c_float * 9)()
        n = C.c_int()
        check(self._L.nfx_batch_tuning(self._h, C.cast(tiles, C.c_void_p), C.cast(ms, C.c_void_p), 9, C.byref(n)))
        nb = C.c_int()
        bt = (C.c_int * 3)()
        bc = (C.c_int64 * 3)()
        bn = (C.c_int64 * 3)()
        check(self._L.nfx_batch_buckets(self._h, 3, C.byref(nb), C.cast(bt, C.c_void_p), C.cast(bc, C.c_void_p),
                                        C.cast(bn, C.c_void_p)))
        return {"cells": a.value, "tets": b.value, "nodes": c.value, "tile_tets": d.value,
                "tuning": [(tiles[i], ms[i]) for i in range(n.value)],
                "buckets": [{"tile_tets": bt[i], "cells": bc[i], "tets": bn[i]} for i in range(nb.value)]}
