"""Algorithm types and ``isosurface``, mirroring Meshing.jl v0.7.0.

* ``AbstractMeshingAlgorithm``      src/algorithmtypes.jl:10
* ``MarchingCubes(iso=0.0)``        src/algorithmtypes.jl:23-25
* ``MarchingTetrahedra(iso=0.0, eps=1e-3)``  src/algorithmtypes.jl:37-40
* ``NaiveSurfaceNets(iso=0.0)``     named in README.md:21; defined by this project
* ``isosurface(A, args...)``        src/isosurface.jl:30-32 (defaults to MarchingCubes())
* ``isosurface(A, method, X=-1:1, Y=-1:1, Z=-1:1)``  src/marching_cubes.jl:27,
  src/marching_tetrahedra.jl:129

Results match the reference: vertex eltype float(FT) with FT the promotion of
the range endpoints, the volume eltype, iso (and eps for MT); faces are
1-based int64 triples; both in the reference's emission order.
"""
import ctypes
import threading
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _lib
from ._lib import (MESH_ALG_MC, MESH_ALG_MT, MESH_ALG_NSN, MESH_DT_F16, MESH_DT_F32, MESH_DT_F64, MESH_DT_I8, MESH_DT_I16,
                   MESH_DT_I32, MESH_DT_I64, MESH_DT_U8, MESH_DT_U16,
                   Context, MeshParams, check)


class AbstractMeshingAlgorithm:
    """Abstract type of an isosurface extraction algorithm (src/algorithmtypes.jl:10)."""


@dataclass(frozen=True)
class MarchingCubes(AbstractMeshingAlgorithm):
    """Marching Cubes; vertices are repeated per cell (src/algorithmtypes.jl:12-25).

    ``weld=True`` (opt-in, no counterpart in the reference) gives one vertex per
    crossed lattice edge: numbered when the edge is first met in the
    reference's emission order, placed by that cell's vertex_interp, with the
    reference's triangles on those ids."""
    iso: Any = 0.0
    weld: bool = False


@dataclass(frozen=True)
class MarchingTetrahedra(AbstractMeshingAlgorithm):
    """Marching Tetrahedra with shared vertices; ``eps`` keeps vertices off
    cell corners (src/algorithmtypes.jl:28-40)."""
    iso: Any = 0.0
    eps: Any = 1e-3


@dataclass(frozen=True)
class NaiveSurfaceNets(AbstractMeshingAlgorithm):
    """Naive Surface Nets (not implemented by the reference; defined here).

    One vertex per cell whose corners straddle ``iso``, placed at the mean of
    the crossing points on the cell's crossed edges (each computed like
    Marching Cubes' vertex_interp); for every crossed lattice edge with four
    surrounding cells, two triangles joining those cells' vertices, oriented
    so that the normal points towards increasing values."""
    iso: Any = 0.0


_ALG = {MarchingCubes: MESH_ALG_MC, MarchingTetrahedra: MESH_ALG_MT, NaiveSurfaceNets: MESH_ALG_NSN}
_VOL_DT = {np.dtype(np.uint16): MESH_DT_U16, np.dtype(np.float32): MESH_DT_F32, np.dtype(np.float64): MESH_DT_F64,
           np.dtype(np.int32): MESH_DT_I32, np.dtype(np.int64): MESH_DT_I64, np.dtype(np.float16): MESH_DT_F16,
           np.dtype(np.int16): MESH_DT_I16, np.dtype(np.int8): MESH_DT_I8, np.dtype(np.uint8): MESH_DT_U8}


def _scalar(v, what):
    """(mesh dtype, value) of a scalar, following the Julia type of the Python value."""
    if isinstance(v, (bool, np.bool_)):
        raise TypeError('%s: Bool is not supported' % what)
    if isinstance(v, np.float32):
        return MESH_DT_F32, float(v)
    if isinstance(v, (float, np.float64)):
        return MESH_DT_F64, float(v)
    if isinstance(v, (int, np.integer)):
        if abs(int(v)) > 2 ** 53:
            raise ValueError('%s: integer beyond 2^53' % what)
        return MESH_DT_I64, float(int(v))
    try:  # 0-d torch tensors / numpy scalars of other kinds
        import torch
        if isinstance(v, torch.Tensor) and v.dim() == 0:
            return _scalar(v.cpu().numpy()[()], what)
    except ImportError:
        pass
    raise TypeError('%s: unsupported scalar type %s' % (what, type(v).__name__))


def _first_last(r, what):
    if isinstance(r, range):
        if len(r) == 0:
            raise ValueError('%s: empty range' % what)
        return r[0], r[-1]
    try:
        return r[0], r[-1]
    except (TypeError, IndexError):
        raise TypeError('%s must be a range, a (first, last) pair or a sequence' % what)


def make_params(method, X=(-1, 1), Y=(-1, 1), Z=(-1, 1)):
    """MeshParams for an algorithm instance and the X, Y, Z arguments."""
    if type(method) not in _ALG:
        raise TypeError('method must be MarchingCubes, MarchingTetrahedra or NaiveSurfaceNets')
    p = MeshParams()
    _lib.load().mesh_params_default(ctypes.byref(p))
    p.alg = _ALG[type(method)]
    if getattr(method, 'weld', False):
        p.alg = _lib.MESH_ALG_MC_WELDED
    p.iso_type, p.iso = _scalar(method.iso, 'iso')
    if isinstance(method, MarchingTetrahedra):
        p.eps_type, p.eps = _scalar(method.eps, 'eps')
        if p.eps_type == MESH_DT_I64:
            raise TypeError('eps must be a Float32 or Float64')
    ends = []
    for r, n in ((X, 'X'), (Y, 'Y'), (Z, 'Z')):
        ends.extend(_first_last(r, n))
    tys = set()
    for i, e in enumerate(ends):
        t, v = _scalar(e, 'range endpoint')
        tys.add(t)
        p.range[i] = v
    if len(tys) != 1:
        raise TypeError('X, Y and Z endpoints must share one type')
    p.range_type = tys.pop()
    return p


def output_float_bits(vol_dtype, method, X=(-1, 1), Y=(-1, 1), Z=(-1, 1)):
    """32 or 64: the bits of float(FT) the reference would return."""
    p = make_params(method, X, Y, Z)
    bits = ctypes.c_int()
    check(_lib.load().mesh_output_float_bits(_VOL_DT[np.dtype(vol_dtype)], ctypes.byref(p), ctypes.byref(bits)))
    return bits.value


_local = threading.local()


def default_context(device=0):
    """The calling thread's context for `device` (a context is not thread-safe)."""
    ctxs = getattr(_local, 'ctxs', None)
    if ctxs is None:
        ctxs = _local.ctxs = {}
    if device not in ctxs:
        ctxs[device] = Context(device)
    return ctxs[device]


def _is_torch(A):
    try:
        import torch
        return isinstance(A, torch.Tensor)
    except ImportError:
        return False


def _torch_julia_layout(t):
    """A view of `t` (indexed [x, y, z]) whose memory is x-fastest."""
    nx, ny, nz = t.shape
    if t.stride() == (1, nx, nx * ny) or t.numel() == 0:
        return t
    return t.permute(2, 1, 0).contiguous().permute(2, 1, 0)


def _split_args(args):
    if args and isinstance(args[0], AbstractMeshingAlgorithm):
        return args[0], args[1:]
    return MarchingCubes(), args  # src/isosurface.jl:30-32


def isosurface(A, *args, ctx=None):
    """isosurface(A[, method][, X, Y, Z]) -> (points, faces).

    ``A``: 3-D numpy array or torch tensor indexed [x, y, z], eltype UInt8, Int8, Int16,
    UInt16, Int32, Int64, Float16, Float32 or Float64.  numpy (and CPU torch) inputs return numpy arrays;
    CUDA torch inputs return CUDA torch tensors: points (V, 3) of float(FT)
    and faces (F, 3) int64, 1-based.
    """
    method, rest = _split_args(args)
    if len(rest) > 3:
        raise TypeError('isosurface takes at most X, Y, Z after the method')
    p = make_params(method, *rest)
    lib = _lib.load()
    if _is_torch(A):
        import torch
        if A.dim() != 3:
            raise ValueError('volume must be 3-D')
        if not A.is_cuda:
            return isosurface(A.numpy(), method, *rest, ctx=ctx)
        dt = _lib.torch_dtype_code(A.dtype)
        if dt is None:
            raise TypeError('unsupported volume eltype %s' % A.dtype)
        t = _torch_julia_layout(A)
        c = ctx or default_context(t.device.index or 0)
        c.follow_torch(t.device)
        nv, nf = ctypes.c_int64(), ctypes.c_int64()
        nx, ny, nz = t.shape
        check(lib.mesh_count(c.handle, ctypes.c_void_p(t.data_ptr()), dt, nx, ny, nz, 1, ctypes.byref(p),
                             ctypes.byref(nv), ctypes.byref(nf)), c.handle)
        bits = ctypes.c_int()
        check(lib.mesh_output_float_bits(dt, ctypes.byref(p), ctypes.byref(bits)))
        ft = torch.float32 if bits.value == 32 else torch.float64
        verts = torch.empty((nv.value, 3), dtype=ft, device=t.device)
        faces = torch.empty((nf.value, 3), dtype=torch.int64, device=t.device)
        check(lib.mesh_fill(c.handle, ctypes.c_void_p(verts.data_ptr()), ctypes.c_void_p(faces.data_ptr()), 1),
              c.handle)
        return verts, faces
    A = np.asarray(A)
    if A.ndim != 3:
        raise ValueError('volume must be 3-D')
    dt = _VOL_DT.get(A.dtype)
    if dt is None:
        raise TypeError('unsupported volume eltype %s' % A.dtype)
    A = np.asfortranarray(A)
    c = ctx or default_context(0)
    c.set_stream(None)
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    nx, ny, nz = A.shape
    check(lib.mesh_count(c.handle, ctypes.c_void_p(A.ctypes.data), dt, nx, ny, nz, 0, ctypes.byref(p),
                         ctypes.byref(nv), ctypes.byref(nf)), c.handle)
    bits = ctypes.c_int()
    check(lib.mesh_output_float_bits(dt, ctypes.byref(p), ctypes.byref(bits)))
    verts = np.empty((nv.value, 3), dtype=np.float32 if bits.value == 32 else np.float64)
    faces = np.empty((nf.value, 3), dtype=np.int64)
    check(lib.mesh_fill(c.handle, ctypes.c_void_p(verts.ctypes.data), ctypes.c_void_p(faces.ctypes.data), 0),
          c.handle)
    return verts, faces


def isosurface_slabs(A, method=None, X=(-1, 1), Y=(-1, 1), Z=(-1, 1), slab_cells=None, slab_bytes=4 << 30,
                     ctx=None):
    """isosurface of a host volume larger than device memory, one x slab at a time.

    x is the outermost axis of the reference's emission order
    (src/marching_cubes.jl:40, src/marching_tetrahedra.jl:144), so the meshes of
    consecutive x slabs of cells, concatenated with face indices offset by the
    vertices before them, are the mesh of the whole volume.  Slab k holds cells
    [c0, c1); its node coordinates are those of the whole volume's LinRange
    (mesh_set_x_window).  Marching Cubes slabs read samples [c0, c1].
    MarchingTetrahedra and NaiveSurfaceNets share vertices between cells: a
    vertex on a slab boundary belongs to the cell column before it (the first
    cell to touch an edge is the lowest one), so every slab after the first
    reads samples [c0 - 1, c1] -- the previous slab's last cell column is its
    halo, counted but not emitted -- and its faces that use the previous slab's
    vertices come back with indices <= 0 before the offset is added.
    ``A`` is a numpy array (or memmap) indexed [x, y, z]; ``slab_cells`` cells
    per slab, or as many as fit ``slab_bytes`` of volume.  Returns numpy
    (points, faces) equal to ``isosurface(A, method, X, Y, Z)``.
    """
    method = method or MarchingCubes()
    if getattr(method, 'weld', False):
        raise TypeError('welded meshes do not split into x slabs')
    halo = not isinstance(method, MarchingCubes)
    p = make_params(method, X, Y, Z)
    dt = _VOL_DT.get(np.dtype(A.dtype))
    if dt is None or A.ndim != 3:
        raise TypeError('3-D volume of a supported eltype expected')
    nx, ny, nz = A.shape
    lib = _lib.load()
    bits = ctypes.c_int()
    check(lib.mesh_output_float_bits(dt, ctypes.byref(p), ctypes.byref(bits)))
    ft = np.float32 if bits.value == 32 else np.float64
    if slab_cells is None:
        plane = ny * nz * A.dtype.itemsize
        slab_cells = max(1, int(slab_bytes // max(plane, 1)) - 1 - (1 if halo else 0))
    c = ctx or default_context(0)
    c.set_stream(None)
    vs, fs, voff = [], [], 0
    try:
        for c0 in range(0, max(nx - 1, 0), slab_cells):
            c1 = min(c0 + slab_cells, nx - 1)
            h = 1 if (halo and c0 > 0) else 0
            s0 = c0 - h   # first sample (the halo column's, after slab 0)
            S = np.asfortranarray(A[s0:c1 + 1])
            check(lib.mesh_set_x_window(c.handle, s0, nx, h), c.handle)
            nv, nf = ctypes.c_int64(), ctypes.c_int64()
            check(lib.mesh_count(c.handle, ctypes.c_void_p(S.ctypes.data), dt, S.shape[0], ny, nz, 0,
                                 ctypes.byref(p), ctypes.byref(nv), ctypes.byref(nf)), c.handle)
            v = np.empty((nv.value, 3), dtype=ft)
            f = np.empty((nf.value, 3), dtype=np.int64)
            check(lib.mesh_fill(c.handle, ctypes.c_void_p(v.ctypes.data), ctypes.c_void_p(f.ctypes.data), 0),
                  c.handle)
            f += voff
            voff += nv.value
            vs.append(v)
            fs.append(f)
    finally:
        lib.mesh_set_x_window(c.handle, 0, 0, 0)
    if not vs:
        return np.empty((0, 3), dtype=ft), np.empty((0, 3), dtype=np.int64)
    return np.concatenate(vs), np.concatenate(fs)


def isosurface_device(A, method=None, X=(-1, 1), Y=(-1, 1), Z=(-1, 1), verts=None, faces=None, counts=None,
                      ctx=None):
    """Device-resident extraction with no host round trip (mesh_extract_device).

    ``A`` is a CUDA tensor in Julia layout; ``verts`` / ``faces`` are
    preallocated CUDA tensors whose first dimension is the capacity; ``counts``
    (int64[2], CUDA) receives (nverts, nfaces).  Work is queued on the current
    torch stream; call ``ctx.sync()``-equivalent ``sync(ctx)`` or synchronize
    the stream before reading.  Returns counts.
    """
    import torch
    method = method or MarchingCubes()
    p = make_params(method, X, Y, Z)
    dt = _lib.torch_dtype_code(A.dtype)
    if dt is None:
        raise TypeError('unsupported volume eltype %s' % A.dtype)
    t = _torch_julia_layout(A)
    c = ctx or default_context(t.device.index or 0)
    c.follow_torch(t.device)
    if counts is None:
        counts = torch.zeros(2, dtype=torch.int64, device=t.device)
    nx, ny, nz = t.shape
    vp = ctypes.c_void_p(verts.data_ptr()) if verts is not None else None
    fp = ctypes.c_void_p(faces.data_ptr()) if faces is not None else None
    check(_lib.load().mesh_extract_device(c.handle, ctypes.c_void_p(t.data_ptr()), dt, nx, ny, nz, ctypes.byref(p),
                                          vp, verts.shape[0] if verts is not None else 0, fp,
                                          faces.shape[0] if faces is not None else 0,
                                          ctypes.c_void_p(counts.data_ptr())), c.handle)
    return counts


def sync(ctx=None, device=0):
    c = ctx or default_context(device)
    check(_lib.load().mesh_ctx_sync(c.handle), c.handle)
