"""Python mirror of solver::FieldRegistry (src/solver/FieldRegistry.hpp:30-80)
with the fields in device memory, and of io::Checkpoint
(src/io/Checkpoint.hpp:41-58): the reference's checkpoint file, written from
and read into the device registry."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check
from .solver import Context, default_context, register_child


class DeviceFieldRegistry:
    """scalar(name, n) / vector(name, n) return device addresses (a vector
    field is one [3][n] array); find() returns (address, n) or (None, -1)."""

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        h = C.c_void_p()
        check(self.L.simall_fields_create(self.ctx.handle, C.byref(h)), self.ctx.handle)
        self.handle = h.value
        register_child(self)
        self.ctx.children.add(self)

    def scalar(self, name: str, n: int) -> int:
        d = C.c_void_p()
        check(self.L.simall_fields_scalar(self.handle, name.encode(), int(n), C.byref(d)), self.ctx.handle)
        return d.value

    def vector(self, name: str, n: int) -> int:
        x = C.c_void_p()
        check(self.L.simall_fields_vector(self.handle, name.encode(), int(n), C.byref(x), None, None),
              self.ctx.handle)
        return x.value

    def find(self, name: str, vector: bool = False):
        d = C.c_void_p()
        n = C.c_int64()
        check(self.L.simall_fields_find(self.handle, name.encode(), int(vector), C.byref(d), C.byref(n)),
              self.ctx.handle)
        return (d.value, n.value) if n.value >= 0 else (None, -1)

    def names(self):
        """(scalar names, vector names) in insertion order."""
        ns, nv = C.c_int(), C.c_int()
        check(self.L.simall_fields_count(self.handle, C.byref(ns), C.byref(nv)))
        out = []
        for vec, cnt in ((0, ns.value), (1, nv.value)):
            lst = []
            for i in range(cnt):
                buf = C.create_string_buffer(512)
                check(self.L.simall_fields_name(self.handle, vec, i, buf, 512, None))
                lst.append(buf.value.decode())
            out.append(lst)
        return tuple(out)

    def upload(self, name: str, values, vector: bool = False):
        """Create / re-size the field from a host array ((n,) or (3, n))."""
        a = np.ascontiguousarray(values, np.float64)
        n = a.shape[-1] if vector else a.size
        if vector and a.shape != (3, n):
            raise ValueError("a vector field is uploaded as a (3, n) array")
        check(self.L.simall_fields_upload(self.handle, name.encode(), int(vector), a.ctypes.data, int(n)),
              self.ctx.handle)

    def download(self, name: str, vector: bool = False) -> np.ndarray:
        _, n = self.find(name, vector)
        if n < 0:
            raise KeyError(name)
        out = np.empty((3, n) if vector else n)
        check(self.L.simall_fields_download(self.handle, name.encode(), int(vector), out.ctypes.data),
              self.ctx.handle)
        return out

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.L.simall_fields_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def checkpoint_write(path: str, mesh: dict, fields: DeviceFieldRegistry, iteration: int = 0, time: float = 0.0,
                     settings_hash: int = 0) -> None:
    """Checkpoint::write: mesh = dict of the 20 mesh SoA arrays
    (_lib.CHECKPOINT_MESH_ARRAYS names) -- nodes, faces, cells."""
    keep = {}
    m = _lib.CheckpointMesh()
    for name, dt in _lib.CHECKPOINT_MESH_ARRAYS:
        a = np.ascontiguousarray(mesh[name], dt)
        keep[name] = a
        setattr(m, name, a.ctypes.data if a.size else None)
    m.n_nodes = len(keep["node_x"])
    m.n_faces = len(keep["owner"])
    m.n_cells = len(keep["volume"])
    m.n_face_nodes = len(keep["face_node_indices"])
    m.n_cell_faces = len(keep["cell_face_indices"])
    if len(keep["face_node_offsets"]) not in (0, m.n_faces + 1) or \
            len(keep["cell_face_offsets"]) not in (0, m.n_cells + 1):
        raise ValueError("offset arrays need n + 1 entries")
    meta = _lib.CheckpointMeta(int(iteration), float(time), int(settings_hash))
    check(fields.L.simall_checkpoint_write(path.encode(), C.byref(m), fields.handle, C.byref(meta)),
          fields.ctx.handle)


def checkpoint_read(path: str, fields: DeviceFieldRegistry, with_mesh: bool = True):
    """Checkpoint::read into the registry; returns ((iteration, time,
    settings_hash), mesh dict or None)."""
    meta = _lib.CheckpointMeta()
    m = _lib.CheckpointMesh()
    check(fields.L.simall_checkpoint_read(path.encode(), fields.handle, C.byref(meta),
                                          C.byref(m) if with_mesh else None), fields.ctx.handle)
    mesh = None
    if with_mesh:
        counts = {"node": m.n_nodes, "face": m.n_faces, "cell": m.n_cells}
        sizes = {"node_x": m.n_nodes, "node_y": m.n_nodes, "node_z": m.n_nodes,
                 "face_node_offsets": m.n_faces + 1, "face_node_indices": m.n_face_nodes,
                 "cell_face_offsets": m.n_cells + 1, "cell_face_indices": m.n_cell_faces,
                 "boundary_zone": m.n_faces, "owner": m.n_faces, "neighbor": m.n_faces}
        mesh = {}
        try:
            for name, dt in _lib.CHECKPOINT_MESH_ARRAYS:
                n = sizes.get(name, counts["cell"] if name in ("volume", "cell_centroid_x", "cell_centroid_y",
                                                               "cell_centroid_z") else counts["face"])
                addr = getattr(m, name)
                mesh[name] = np.ctypeslib.as_array(C.cast(addr, C.POINTER(np.ctypeslib.as_ctypes_type(
                    np.dtype(dt)))), (n,)).copy() if (addr and n > 0) else np.zeros(0, dt)
        finally:
            fields.L.simall_checkpoint_mesh_free(C.byref(m))
    return (meta.iteration, meta.time, meta.settings_hash), mesh
