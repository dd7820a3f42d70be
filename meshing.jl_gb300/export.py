"""Mesh export and post-processing: vertex normals on the device, PLY files.

Meshing.jl returns (vertices, faces) and leaves output to other packages (its
etc/output_comparison.jl writes the meshes of the three algorithms to one PLY
file through FileIO).  Here:

    n = vertex_normals(verts, faces)             # CUDA tensors -> (V, 3) unit normals
    write_ply('surface.ply', verts, faces, n)    # binary little-endian PLY
    v, f, n = read_ply('surface.ply')            # numpy, faces 1-based again

``vertex_normals`` is the area-weighted rule of GeometryBasics'
``normals(vertices, faces)``: normal i = normalize(sum of cross(v2 - v1,
v3 - v1) over the faces using vertex i), summed in Float64 on the device
(mesh_vertex_normals in include/meshing_gb300.h).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check


def vertex_normals(verts, faces, ctx=None):
    """Unit vertex normals (V, 3) of a mesh given as CUDA tensors: verts (V, 3)
    float32 / float64, faces (F, 3) int64 1-based.  Returns a CUDA tensor of the
    vertex dtype, computed on the current torch stream."""
    import torch
    from .api import default_context
    if not (verts.is_cuda and faces.is_cuda):
        raise TypeError('vertex_normals takes CUDA tensors')
    if verts.dtype not in (torch.float32, torch.float64) or faces.dtype != torch.int64:
        raise TypeError('verts must be float32 / float64 and faces int64')
    if verts.dim() != 2 or verts.shape[-1] != 3 or faces.dim() != 2 or faces.shape[-1] != 3:
        raise ValueError('verts and faces must be (n, 3)')
    v = verts.contiguous()
    f = faces.contiguous()
    out = torch.empty_like(v)
    c = ctx or default_context(v.device.index or 0)
    c.follow_torch(v.device)
    bits = 32 if v.dtype == torch.float32 else 64
    lib = _lib.load()
    check(lib.mesh_vertex_normals(c.handle, ctypes.c_void_p(v.data_ptr()), bits, v.shape[0],
                                  ctypes.c_void_p(f.data_ptr()), f.shape[0], ctypes.c_void_p(out.data_ptr())),
          c.handle)
    check(lib.mesh_ctx_sync(c.handle), c.handle)
    return out


def _np(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(a)


def write_ply(path, verts, faces, normals=None, binary=True):
    """Writes a triangle mesh (faces 1-based, as isosurface returns them) as a PLY
    file with 0-based int32 vertex indices; float32 / float64 vertex properties
    follow the vertex dtype."""
    v = _np(verts)
    f = _np(faces).astype(np.int64) - 1
    n = None if normals is None else _np(normals).astype(v.dtype)
    if v.dtype not in (np.float32, np.float64):
        raise TypeError('vertices must be float32 or float64')
    if len(f) and (f.min() < 0 or f.max() >= len(v)):
        raise ValueError('face index outside the vertex list')
    if len(f) and f.max() > np.iinfo(np.int32).max:
        raise ValueError('more vertices than int32 PLY indices can address')
    ptype = 'float' if v.dtype == np.float32 else 'double'
    props = ['x', 'y', 'z'] + (['nx', 'ny', 'nz'] if n is not None else [])
    head = ['ply', 'format %s 1.0' % ('binary_little_endian' if binary else 'ascii'),
            'comment meshing_gb300 isosurface', 'element vertex %d' % len(v)]
    head += ['property %s %s' % (ptype, p) for p in props]
    head += ['element face %d' % len(f), 'property list uchar int vertex_indices', 'end_header']
    with open(path, 'wb') as fh:
        fh.write(('\n'.join(head) + '\n').encode('ascii'))
        if binary:
            vt = np.dtype([(p, v.dtype.newbyteorder('<')) for p in props])
            rec = np.empty(len(v), dtype=vt)
            for i, p in enumerate(props[:3]):
                rec[p] = v[:, i]
            if n is not None:
                for i, p in enumerate(props[3:]):
                    rec[p] = n[:, i]
            fh.write(rec.tobytes())
            ft = np.dtype([('n', 'u1'), ('i', '<i4', (3,))])
            fr = np.empty(len(f), dtype=ft)
            fr['n'] = 3
            fr['i'] = f
            fh.write(fr.tobytes())
        else:
            cols = v if n is None else np.concatenate([v, n], axis=1)
            for row in cols:
                fh.write((' '.join(repr(float(x)) for x in row) + '\n').encode('ascii'))
            for row in f:
                fh.write(('3 %d %d %d\n' % tuple(row)).encode('ascii'))
    return path


def read_ply(path):
    """(verts, faces 1-based, normals or None) of a PLY file written by write_ply
    (binary little-endian or ascii triangle meshes)."""
    with open(path, 'rb') as fh:
        if fh.readline().strip() != b'ply':
            raise ValueError('not a PLY file')
        fmt, nv, nf, props, ptype = None, 0, 0, [], None
        elem = None
        while True:
            line = fh.readline().decode('ascii').strip()
            if line == 'end_header':
                break
            w = line.split()
            if not w or w[0] == 'comment':
                continue
            if w[0] == 'format':
                fmt = w[1]
            elif w[0] == 'element':
                elem = w[1]
                if elem == 'vertex':
                    nv = int(w[2])
                elif elem == 'face':
                    nf = int(w[2])
            elif w[0] == 'property' and elem == 'vertex':
                props.append(w[2])
                ptype = w[1]
        dt = np.float32 if ptype in ('float', 'float32') else np.float64
        if fmt == 'binary_little_endian':
            vt = np.dtype([(p, np.dtype(dt).newbyteorder('<')) for p in props])
            rec = np.frombuffer(fh.read(vt.itemsize * nv), dtype=vt)
            fr = np.frombuffer(fh.read(13 * nf), dtype=np.dtype([('n', 'u1'), ('i', '<i4', (3,))]))
            if nf and not (fr['n'] == 3).all():
                raise ValueError('only triangle faces are read')
            cols = np.stack([rec[p] for p in props], axis=1).astype(dt) if nv else np.empty((0, len(props)), dt)
            faces = fr['i'].astype(np.int64) + 1
        elif fmt == 'ascii':
            body = fh.read().decode('ascii').split('\n')
            cols = np.array([[float(x) for x in body[i].split()] for i in range(nv)], dtype=dt).reshape(nv, len(props))
            faces = np.array([[int(x) for x in body[nv + i].split()[1:4]] for i in range(nf)],
                             dtype=np.int64).reshape(nf, 3) + 1
        else:
            raise ValueError('PLY format %r is not read' % fmt)
    verts = np.ascontiguousarray(cols[:, :3])
    normals = np.ascontiguousarray(cols[:, 3:6]) if len(props) >= 6 else None
    return verts, faces, normals


__all__ = ['vertex_normals', 'write_ply', 'read_ply']
