"""Serving loop: continuous batching of isosurface requests (mesh_server_*).

Each request names a volume (a CUDA tensor, or a host array the server uploads
into its pool) and an algorithm; the server answers with
exactly the mesh ``isosurface(A, method, X, Y, Z)`` returns for it alone, kept
resident on the device until released.

    srv = Server(budget_bytes=8 << 30)
    rid = srv.submit(A, MarchingCubes(iso=np.float32(0)))
    verts, faces = srv.result(rid)   # waits; CUDA tensor views into the pool
    srv.release(rid)
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import MESH_DT_F32, MESH_DT_F64, MESH_DT_U16, MeshError
from .api import _VOL_DT, MarchingCubes, _torch_julia_layout, make_params
from .batch import _DeviceArray

STATE = {0: 'queued', 1: 'running', 2: 'done', 3: 'failed'}


def _is_cuda_tensor(A):
    try:
        import torch
    except ImportError:
        return False
    return isinstance(A, torch.Tensor) and A.is_cuda


class Server:
    """A serving loop on CUDA device `device` with a device pool of
    `budget_bytes`, `slots` waves in flight, at most `max_wave` requests per
    wave and `max_queue` waiting requests."""

    def __init__(self, budget_bytes, slots=2, max_wave=256, max_queue=1 << 20, device=0):
        self._lib = _lib.load()
        self.handle = ctypes.c_void_p()
        self._check(self._lib.mesh_server_create(device, int(budget_bytes), slots, max_wave, max_queue,
                                                 ctypes.byref(self.handle)))
        self.device = device
        self._live = {}  # id -> (volume kept alive, float bits)

    def _check(self, rc):
        if rc != 0:
            msg = ''
            if getattr(self, 'handle', None):
                raw = self._lib.mesh_server_last_error(self.handle)
                msg = raw.decode() if raw else ''
            raise MeshError(rc, msg)

    def close(self):
        if self.handle:
            self._lib.mesh_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, A, method=None, X=(-1, 1), Y=(-1, 1), Z=(-1, 1)):
        """Queue isosurface(A, method, X, Y, Z); returns the request id.

        A: a 3-D CUDA tensor (read in place), or a numpy array / CPU tensor
        indexed [x, y, z], which the server uploads into its pool when the
        request is admitted (kept referenced here until the request is released)."""
        method = method or MarchingCubes()
        p = make_params(method, X, Y, Z)
        if _is_cuda_tensor(A):
            import torch
            dt = _lib.torch_dtype_code(A.dtype)
            if dt is None or A.dim() != 3:
                raise TypeError('volume must be a 3-D tensor of a supported eltype')
            t = _torch_julia_layout(A)
            # the server reads the volume on its own streams: finish writing it first
            torch.cuda.current_stream(t.device).synchronize()
            ptr, shape, on_device = t.data_ptr(), tuple(t.shape), 1
        else:
            t = np.asfortranarray(A.numpy() if hasattr(A, 'numpy') else np.asarray(A))
            dt = _VOL_DT.get(t.dtype)
            if dt is None or t.ndim != 3:
                raise TypeError('volume must be a 3-D array of a supported eltype')
            ptr, shape, on_device = t.ctypes.data, t.shape, 0
        bits = ctypes.c_int()
        self._check(self._lib.mesh_output_float_bits(dt, ctypes.byref(p), ctypes.byref(bits)))
        rid = ctypes.c_int64()
        nx, ny, nz = shape
        self._check(self._lib.mesh_server_submit(self.handle, ctypes.c_void_p(ptr), dt, nx, ny, nz, on_device,
                                                 ctypes.byref(p), ctypes.byref(rid)))
        self._live[rid.value] = (t, bits.value)
        return rid.value

    def _query(self, fn, rid, *extra):
        st, nv, nf = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64()
        v, f = ctypes.c_void_p(), ctypes.c_void_p()
        rc = fn(self.handle, rid, *extra, ctypes.byref(st), ctypes.byref(nv), ctypes.byref(nf), ctypes.byref(v),
                ctypes.byref(f))
        self._check(rc)
        return st.value, nv.value, nf.value, v.value, f.value

    def poll(self, rid):
        """'queued', 'running', 'done' (or MeshError if the request failed)."""
        return STATE[self._query(self._lib.mesh_server_poll, rid)[0]]

    def wait(self, rid, timeout=60.0):
        st = self._query(self._lib.mesh_server_wait, rid, int(timeout * 1e6))[0]
        return STATE[st]

    def result(self, rid, timeout=60.0):
        """(verts, faces) as CUDA tensor views of the request's resident mesh."""
        import torch
        st, nv, nf, v, f = self._query(self._lib.mesh_server_wait, rid, int(timeout * 1e6))
        if st != 2:
            raise TimeoutError('request %d is %s' % (rid, STATE[st]))
        bits = self._live[rid][1]
        dev = torch.device('cuda', self.device)
        ft = torch.float32 if bits == 32 else torch.float64
        verts = torch.as_tensor(_DeviceArray(v, (nv, 3), '<f4' if bits == 32 else '<f8'), device=dev) if nv else \
            torch.empty((0, 3), dtype=ft, device=dev)
        faces = torch.as_tensor(_DeviceArray(f, (nf, 3), '<i8'), device=dev) if nf else \
            torch.empty((0, 3), dtype=torch.int64, device=dev)
        return verts, faces

    def release(self, rid):
        self._check(self._lib.mesh_server_release(self.handle, rid))
        self._live.pop(rid, None)

    def replay(self, reqs, arrivals):
        """Native load generator: request i = (A, method, (X, Y, Z)) is submitted
        arrivals[i] seconds after the start and released as soon as it ends;
        returns when all have ended (see stats())."""
        import torch
        n = len(reqs)
        vols = (ctypes.c_void_p * n)()
        dts = (ctypes.c_int * n)()
        dims = (ctypes.c_int64 * (3 * n))()
        prms = (_lib.MeshParams * n)()
        keep = []
        for i, (A, m, r) in enumerate(reqs):
            t = _torch_julia_layout(A)
            keep.append(t)
            vols[i] = t.data_ptr()
            dts[i] = _lib.torch_dtype_code(t.dtype)
            dims[3 * i:3 * i + 3] = list(t.shape)
            prms[i] = make_params(m, *r)
        torch.cuda.synchronize()
        arr = (ctypes.c_double * n)(*[float(x) for x in arrivals])
        self._check(self._lib.mesh_server_replay(self.handle, n, vols, dts, dims, prms, arr))

    def stats(self):
        st = (ctypes.c_double * 14)()
        self._check(self._lib.mesh_server_stats(self.handle, st))
        keys = ('completed', 'rejected', 'failed', 'p50_ms', 'p99_ms', 'mean_ms', 'samples', 'wall_s',
                'peak_reserved_bytes', 'pool_bytes', 'queued', 'reserved_bytes', 'waves', 'requests_per_wave')
        return dict(zip(keys, list(st)))

    def reset_stats(self):
        self._check(self._lib.mesh_server_reset_stats(self.handle))
