"""Batched Marching Cubes: many CUDA volumes of uneven shape in one pass.

Each volume of a batch gives exactly what ``isosurface(A_i, MarchingCubes(iso),
X_i, Y_i, Z_i)`` gives on it alone (src/marching_cubes.jl:27-64); the batch runs
every stage once over all volumes instead of one launch sequence per volume
(``mesh_batch_*`` in include/meshing_gb300.h).

    b = Batch([A1, A2, ...], MarchingCubes(iso=np.float32(0)), (-1, 1), (-1, 1), (-1, 1))
    b.count()                  # sizes the outputs
    b.set_graph(True)          # replay the run from a CUDA graph
    b.run(); b.sync()
    verts, faces = b.volume(i)  # views into the concatenated outputs
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import MESH_DT_F32, MESH_DT_F64, MESH_DT_U16, check
from .api import MarchingCubes, _torch_julia_layout, default_context, make_params


class _DeviceArray:
    """A device buffer seen by torch.as_tensor (zero copy)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {'data': (int(ptr), False), 'shape': tuple(shape), 'typestr': typestr,
                                         'version': 3, 'strides': None}


class Batch:
    """Marching Cubes over CUDA volumes ``volumes`` (3-D tensors indexed [x, y, z],
    one dtype).  ``X, Y, Z`` apply to every volume, or ``ranges`` gives one
    (X, Y, Z) per volume (endpoints of one type)."""

    def __init__(self, volumes, method=None, X=(-1, 1), Y=(-1, 1), Z=(-1, 1), ranges=None, ctx=None):
        import torch
        method = method or MarchingCubes()
        if not isinstance(method, MarchingCubes):
            raise TypeError('batches run MarchingCubes only')
        if not volumes:
            raise ValueError('empty batch')
        dt = _lib.torch_dtype_code(volumes[0].dtype)
        if dt is None or any(v.dtype != volumes[0].dtype or v.dim() != 3 or not v.is_cuda for v in volumes):
            raise TypeError('volumes must be 3-D CUDA tensors of one dtype (UInt16, Int32, Int64, Float32 or Float64)')
        self._vols = [_torch_julia_layout(v) for v in volumes]  # keeps the memory alive
        self.device = self._vols[0].device
        self.ctx = ctx or default_context(self.device.index or 0)
        self.ctx.follow_torch(self.device)
        self.params = make_params(method, X, Y, Z)
        n = len(self._vols)
        rng = None
        if ranges is not None:
            if len(ranges) != n:
                raise ValueError('one (X, Y, Z) per volume')
            ps = [make_params(method, *r) for r in ranges]
            if any(q.range_type != ps[0].range_type for q in ps):
                raise TypeError('range endpoints of all volumes must share one type')
            self.params.range_type = ps[0].range_type
            rng = (ctypes.c_double * (6 * n))(*[q.range[k] for q in ps for k in range(6)])
        ptrs = (ctypes.c_void_p * n)(*[v.data_ptr() for v in self._vols])
        dims = (ctypes.c_int64 * (3 * n))(*[s for v in self._vols for s in v.shape])
        self._lib = _lib.load()
        self.handle = ctypes.c_void_p()
        check(self._lib.mesh_batch_create(self.ctx.handle, n, ptrs, dt, dims, ctypes.byref(self.params), rng,
                                          ctypes.byref(self.handle)), self.ctx.handle)
        self.n = n
        bits = ctypes.c_int()
        check(self._lib.mesh_output_float_bits(dt, ctypes.byref(self.params), ctypes.byref(bits)))
        self.float_bits = bits.value
        self.nverts = self.nfaces = None

    def close(self):
        if self.handle:
            self._lib.mesh_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def count(self):
        nv, nf = ctypes.c_int64(), ctypes.c_int64()
        check(self._lib.mesh_batch_count(self.handle, ctypes.byref(nv), ctypes.byref(nf)), self.ctx.handle)
        self.nverts, self.nfaces = nv.value, nf.value
        return self.nverts, self.nfaces

    def run(self):
        check(self._lib.mesh_batch_run(self.handle), self.ctx.handle)

    def sync(self):
        check(self._lib.mesh_batch_sync(self.handle), self.ctx.handle)

    def set_graph(self, enable=True):
        check(self._lib.mesh_batch_set_graph(self.handle, 1 if enable else 0), self.ctx.handle)

    @property
    def knobs(self):
        k = (ctypes.c_int * 4)()
        check(self._lib.mesh_batch_knobs(self.handle, k))
        return {'zs': k[0], 'classify_ctas': k[1], 'compact_ctas': k[2], 'scan_threads': k[3]}

    def set_knobs(self, zs=0, classify_ctas=0, compact_ctas=0, scan_threads=1024):
        k = (ctypes.c_int * 4)(zs, classify_ctas, compact_ctas, scan_threads)
        check(self._lib.mesh_batch_set_knobs(self.handle, k), self.ctx.handle)

    def tune(self, reps=3):
        """Autotune the knobs on this batch; returns the tuner's report."""
        buf = ctypes.create_string_buffer(4096)
        check(self._lib.mesh_batch_tune(self.handle, reps, buf, len(buf)), self.ctx.handle)
        self.count()
        return buf.value.decode()

    def outputs(self):
        """(verts [V,3], faces [F,3] int64 1-based per volume, offsets [n+1,2]) as CUDA tensors."""
        import torch
        v, f, o = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        check(self._lib.mesh_batch_outputs(self.handle, ctypes.byref(v), ctypes.byref(f), ctypes.byref(o)),
              self.ctx.handle)
        ft = '<f4' if self.float_bits == 32 else '<f8'
        dev = self.device
        verts = torch.as_tensor(_DeviceArray(v.value, (self.nverts, 3), ft), device=dev) if self.nverts else \
            torch.empty((0, 3), dtype=torch.float32 if self.float_bits == 32 else torch.float64, device=dev)
        faces = torch.as_tensor(_DeviceArray(f.value, (self.nfaces, 3), '<i8'), device=dev) if self.nfaces else \
            torch.empty((0, 3), dtype=torch.int64, device=dev)
        offs = torch.as_tensor(_DeviceArray(o.value, (self.n + 1, 2), '<i8'), device=dev)
        return verts, faces, offs

    def volume(self, i, outputs=None, offsets=None):
        """Vertices and faces of volume i (views)."""
        verts, faces, offs = outputs or self.outputs()
        o = offsets if offsets is not None else offs.cpu().numpy()
        return verts[o[i, 0]:o[i + 1, 0]], faces[o[i, 1]:o[i + 1, 1]]
