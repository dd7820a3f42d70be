"""ctypes wrapper of the C oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, and only as the checker / CPU baseline.  The
product (``meshing.jl_gb300``) never imports it.

Volumes follow Julia's memory layout: an array ``A`` with ``size(A) == (nx, ny, nz)``
is a numpy array of shape (nx, ny, nz) in Fortran order (x fastest).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'liborc.so')
SRC = [os.path.join(HERE, 'oracle.c'), os.path.join(HERE, 'ref_luts.h')]

U16, F32, F64, I64, I32, F16, I16, I8, U8 = 1, 2, 3, 4, 5, 6, 7, 8, 9
ALGS = {'mc': 0, 'mt': 1, 'nsn': 2, 'mcw': 3}
DTYPES = {np.dtype(np.uint16): U16, np.dtype(np.float32): F32, np.dtype(np.float64): F64, np.dtype(np.int64): I64,
          np.dtype(np.int32): I32, np.dtype(np.float16): F16, np.dtype(np.int16): I16, np.dtype(np.int8): I8,
          np.dtype(np.uint8): U8}


def build(force=False):
    """Compile oracle.c into _build/liborc.so (no FMA contraction, as the reference)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in SRC):
        return LIB
    tmp = LIB + '.%d.tmp' % os.getpid()
    subprocess.check_call(['gcc', '-O2', '-std=c11', '-fPIC', '-shared', '-ffp-contract=off', '-fno-fast-math',
                           '-o', tmp, os.path.join(HERE, 'oracle.c'), '-lm'])
    os.replace(tmp, LIB)
    return LIB


class _Mesh(ctypes.Structure):
    _fields_ = [('verts', ctypes.c_void_p), ('nverts', ctypes.c_int64), ('faces', ctypes.c_void_p),
                ('nfaces', ctypes.c_int64), ('out_bits', ctypes.c_int), ('cap_v', ctypes.c_int64),
                ('cap_f', ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.orc_isosurface.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_Mesh)]
        _lib.orc_isosurface.restype = ctypes.c_int
        _lib.orc_isosurface_mc_xwin.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                                ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(_Mesh)]
        _lib.orc_isosurface_mc_xwin.restype = ctypes.c_int
        _lib.orc_free.argtypes = [ctypes.POINTER(_Mesh)]
        _lib.orc_output_bits.argtypes = [ctypes.c_int] * 5
        _lib.orc_cubeindex.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_double]
        _lib.orc_vertex_interp_f64.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                                               ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        _lib.orc_linrange_at.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                                         ctypes.c_int64]
        _lib.orc_linrange_at.restype = ctypes.c_double
    return _lib


def scalar_type(v):
    """Julia eltype of a Python/numpy scalar: int -> Int64, float -> Float64."""
    if isinstance(v, (np.float32,)):
        return F32
    if isinstance(v, (float, np.float64)):
        return F64
    if isinstance(v, (bool, np.bool_)):
        raise TypeError('Bool iso/eps is not supported')
    if isinstance(v, (int, np.integer)):
        return I64
    raise TypeError('unsupported scalar %r' % (v,))


def isosurface(vol, alg='mc', iso=0.0, eps=1e-3, ranges=((-1, 1), (-1, 1), (-1, 1))):
    """Run the oracle.  ``vol``: numpy (nx, ny, nz) Fortran-ordered array.

    iso / eps / range endpoints carry their Julia type through their Python
    type (int -> Int64, float -> Float64, np.float32 -> Float32).
    Returns (verts (V,3) float32|float64, faces (F,3) int64, 1-based).
    """
    vol = np.asfortranarray(vol)
    T = DTYPES[vol.dtype]
    nx, ny, nz = (vol.shape + (1, 1, 1))[:3] if vol.ndim == 3 else (0, 0, 0)
    rt = {scalar_type(ranges[a][b]) for a in range(3) for b in range(2)}
    if len(rt) != 1:
        raise TypeError('all range endpoints must share one type')
    R = rt.pop()
    rg = (ctypes.c_double * 6)(*[float(ranges[a][b]) for a in range(3) for b in range(2)])
    m = _Mesh()
    rc = lib().orc_isosurface(vol.ctypes.data, T, nx, ny, nz, ALGS[alg], scalar_type(iso), float(iso),
                              scalar_type(eps), float(eps), R, rg, ctypes.byref(m))
    if rc:
        raise RuntimeError('oracle failed with status %d' % rc)
    return _take(m)


def _range_args(ranges):
    rt = {scalar_type(ranges[a][b]) for a in range(3) for b in range(2)}
    if len(rt) != 1:
        raise TypeError('all range endpoints must share one type')
    return rt.pop(), (ctypes.c_double * 6)(*[float(ranges[a][b]) for a in range(3) for b in range(2)])


def mc_xwindow(vol, x0, x1, iso=0.0, ranges=((-1, 1), (-1, 1), (-1, 1))):
    """MarchingCubes over the cells x0 .. x1-1 of ``vol`` (Fortran-ordered),
    with the whole volume's LinRange node coordinates.  Returns the block of the
    whole mesh that those cells emit, faces numbered from 1 within the block."""
    if not vol.flags['F_CONTIGUOUS']:
        raise ValueError('vol must be Fortran-ordered')
    nx, ny, nz = vol.shape
    R, rg = _range_args(ranges)
    m = _Mesh()
    rc = lib().orc_isosurface_mc_xwin(vol.ctypes.data, DTYPES[vol.dtype], nx, ny, nz, x0, x1, scalar_type(iso),
                                      float(iso), R, rg, ctypes.byref(m))
    if rc:
        raise RuntimeError('oracle failed with status %d' % rc)
    return _take(m)


def mc_xwindows(vol, iso=0.0, ranges=((-1, 1), (-1, 1), (-1, 1)), windows=64, threads=None):
    """The whole MarchingCubes mesh of ``vol`` as consecutive x-window blocks,
    meshed on several threads (the C oracle runs without the GIL).  Returns a
    list of (x0, x1, verts, faces) in emission order."""
    from concurrent.futures import ThreadPoolExecutor
    vol = np.asfortranarray(vol)
    cx = vol.shape[0] - 1
    cuts = sorted({round(i * cx / windows) for i in range(windows + 1)})
    spans = list(zip(cuts[:-1], cuts[1:]))
    threads = threads or max(1, min(len(spans), os.cpu_count() or 1))
    with ThreadPoolExecutor(threads) as ex:
        meshes = list(ex.map(lambda s: mc_xwindow(vol, s[0], s[1], iso, ranges), spans))
    return [(a, b, v, f) for (a, b), (v, f) in zip(spans, meshes)]


def _take(m):
    """numpy copies of an orc_mesh's arrays; frees the mesh."""
    try:
        ft = np.float32 if m.out_bits == 32 else np.float64
        if m.nverts:
            buf = (ctypes.c_char * (m.nverts * 3 * np.dtype(ft).itemsize)).from_address(m.verts)
            verts = np.frombuffer(buf, dtype=ft).reshape(-1, 3).copy()
        else:
            verts = np.zeros((0, 3), ft)
        if m.nfaces:
            buf = (ctypes.c_char * (m.nfaces * 24)).from_address(m.faces)
            faces = np.frombuffer(buf, dtype=np.int64).reshape(-1, 3).copy()
        else:
            faces = np.zeros((0, 3), np.int64)
    finally:
        lib().orc_free(ctypes.byref(m))
    return verts, faces


def output_bits(dtype, alg, iso, eps=1e-3, range_type=I64):
    return lib().orc_output_bits(DTYPES[np.dtype(dtype)], ALGS[alg], scalar_type(iso), scalar_type(eps), range_type)


def cubeindex(vals, iso):
    arr = (ctypes.c_double * 8)(*[float(v) for v in vals])
    return lib().orc_cubeindex(arr, float(iso))


def vertex_interp(iso, p1, p2, v1, v2):
    a = (ctypes.c_double * 3)(*map(float, p1))
    b = (ctypes.c_double * 3)(*map(float, p2))
    out = (ctypes.c_double * 3)()
    lib().orc_vertex_interp_f64(float(iso), a, b, float(v1), float(v2), out)
    return tuple(out)


def linrange_at(L, a, b, n, i):
    return lib().orc_linrange_at(L, a, b, n, i)
