"""ctypes binding of the C ABI declared in include/meshing_gb300.h.

Loads ``_build/libmeshing_gb300.so``.  There is no fallback: if the library is
missing or cannot be loaded, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_build', 'libmeshing_gb300.so')

MESH_DT_U16, MESH_DT_F32, MESH_DT_F64, MESH_DT_I64, MESH_DT_I32, MESH_DT_F16 = 1, 2, 3, 4, 5, 6
MESH_DT_I16, MESH_DT_I8, MESH_DT_U8 = 7, 8, 9
MESH_ALG_MC, MESH_ALG_MT, MESH_ALG_NSN, MESH_ALG_MC_WELDED = 0, 1, 2, 3
STATUS = {0: 'MESH_OK', 1: 'MESH_EINVAL', 2: 'MESH_ENOMEM', 3: 'MESH_ECUDA', 4: 'MESH_EDEVICE', 5: 'MESH_ESTATE',
          6: 'MESH_ECAPACITY', 7: 'MESH_ETOOLARGE', 8: 'MESH_ESCRATCH', 9: 'MESH_EBUDGET', 10: 'MESH_EBUSY'}

# every symbol the header declares
EXPORTS = ('mesh_params_default', 'mesh_ctx_create', 'mesh_ctx_destroy', 'mesh_ctx_set_stream', 'mesh_set_x_window',
           'mesh_status_string',
           'mesh_ctx_last_error', 'mesh_output_float_bits', 'mesh_count', 'mesh_fill', 'mesh_extract_device',
           'mesh_ctx_sync', 'mesh_ctx_enable_timing', 'mesh_ctx_stage_times', 'mesh_extract_noalloc',
           'mesh_vertex_normals',
           'mesh_batch_create', 'mesh_batch_destroy', 'mesh_batch_count', 'mesh_batch_run', 'mesh_batch_sync',
           'mesh_batch_outputs', 'mesh_batch_set_graph', 'mesh_batch_set_knobs', 'mesh_batch_knobs', 'mesh_batch_tune',
           'mesh_server_create', 'mesh_server_destroy', 'mesh_server_last_error', 'mesh_server_submit',
           'mesh_server_poll', 'mesh_server_wait', 'mesh_server_release', 'mesh_server_stats',
           'mesh_server_reset_stats', 'mesh_server_replay')


class MeshParams(ctypes.Structure):
    _fields_ = [('alg', ctypes.c_int32), ('iso_type', ctypes.c_int32), ('iso', ctypes.c_double),
                ('eps_type', ctypes.c_int32), ('eps', ctypes.c_double), ('range_type', ctypes.c_int32),
                ('range', ctypes.c_double * 6)]


class MeshError(RuntimeError):
    def __init__(self, status, message=''):
        self.status = status
        super().__init__('%s: %s' % (STATUS.get(status, status), message))


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError('meshing_gb300 CUDA library not built (%s); call __graft_entry__.build() or '
                           'python meshing.jl_gb300/_build.py' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    vp, i64, c_int = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    sig = {
        'mesh_params_default': (None, [P(MeshParams)]),
        'mesh_ctx_create': (c_int, [c_int, P(vp)]),
        'mesh_ctx_destroy': (None, [vp]),
        'mesh_ctx_set_stream': (c_int, [vp, vp]),
        'mesh_set_x_window': (c_int, [vp, ctypes.c_int64, ctypes.c_int64, c_int]),
        'mesh_vertex_normals': (c_int, [vp, vp, c_int, ctypes.c_int64, vp, ctypes.c_int64, vp]),
        'mesh_status_string': (ctypes.c_char_p, [c_int]),
        'mesh_ctx_last_error': (ctypes.c_char_p, [vp]),
        'mesh_output_float_bits': (c_int, [c_int, P(MeshParams), P(c_int)]),
        'mesh_count': (c_int, [vp, vp, c_int, i64, i64, i64, c_int, P(MeshParams), P(i64), P(i64)]),
        'mesh_fill': (c_int, [vp, vp, vp, c_int]),
        'mesh_extract_device': (c_int, [vp, vp, c_int, i64, i64, i64, P(MeshParams), vp, i64, vp, i64, vp]),
        'mesh_ctx_sync': (c_int, [vp]),
        'mesh_ctx_enable_timing': (c_int, [vp, c_int]),
        'mesh_ctx_stage_times': (c_int, [vp, P(ctypes.c_double), P(i64)]),
        'mesh_extract_noalloc': (c_int, [vp, c_int, i64, i64, i64, P(MeshParams), vp, i64, vp, i64, vp, vp]),
        'mesh_batch_create': (c_int, [vp, c_int, P(vp), c_int, P(i64), P(MeshParams), P(ctypes.c_double), P(vp)]),
        'mesh_batch_destroy': (None, [vp]),
        'mesh_batch_count': (c_int, [vp, P(i64), P(i64)]),
        'mesh_batch_run': (c_int, [vp]),
        'mesh_batch_sync': (c_int, [vp]),
        'mesh_batch_outputs': (c_int, [vp, P(vp), P(vp), P(vp)]),
        'mesh_batch_set_graph': (c_int, [vp, c_int]),
        'mesh_batch_set_knobs': (c_int, [vp, P(c_int)]),
        'mesh_batch_knobs': (c_int, [vp, P(c_int)]),
        'mesh_batch_tune': (c_int, [vp, c_int, ctypes.c_char_p, c_int]),
        'mesh_server_create': (c_int, [c_int, i64, c_int, c_int, c_int, P(vp)]),
        'mesh_server_destroy': (None, [vp]),
        'mesh_server_last_error': (ctypes.c_char_p, [vp]),
        'mesh_server_submit': (c_int, [vp, vp, c_int, i64, i64, i64, c_int, P(MeshParams), P(i64)]),
        'mesh_server_poll': (c_int, [vp, i64, P(c_int), P(i64), P(i64), P(vp), P(vp)]),
        'mesh_server_wait': (c_int, [vp, i64, i64, P(c_int), P(i64), P(i64), P(vp), P(vp)]),
        'mesh_server_release': (c_int, [vp, i64]),
        'mesh_server_stats': (c_int, [vp, P(ctypes.c_double)]),
        'mesh_server_reset_stats': (c_int, [vp]),
        'mesh_server_replay': (c_int, [vp, c_int, P(vp), P(c_int), P(i64), P(MeshParams), P(ctypes.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, ctx=None):
    if rc != 0:
        msg = ''
        if ctx:
            raw = load().mesh_ctx_last_error(ctx)
            msg = raw.decode() if raw else ''
        raise MeshError(rc, msg)


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream


class Context:
    """Owns a mesh_ctx (device scratch, stream) for one CUDA device."""

    def __init__(self, device=0):
        self._lib = load()
        h = ctypes.c_void_p()
        check(self._lib.mesh_ctx_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self._lib.mesh_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def enable_timing(self, on=True):
        check(self._lib.mesh_ctx_enable_timing(self.handle, 1 if on else 0), self.handle)

    def stage_times(self):
        """{stage: (total device ms, kernel launches)} since the last query; stages are
        classify (with MESHING_GB300_ONE_WALK=1, the Marching Cubes walk that also
        lists the active cells), scan, emit (MC: vertices and faces straight from
        the volume, or with MESHING_GB300_LIST_EMIT=1 the compaction of the active
        cells by a second walk; MT/NSN: the whole emit), expand (MC list form only:
        active cells into vertices and faces)."""
        ms = (ctypes.c_double * 4)()
        n = (ctypes.c_int64 * 4)()
        check(self._lib.mesh_ctx_stage_times(self.handle, ms, n), self.handle)
        return {k: (ms[i], n[i]) for i, k in enumerate(('classify', 'scan', 'emit', 'expand'))}

    def sync(self):
        check(self._lib.mesh_ctx_sync(self.handle), self.handle)

    def set_stream(self, stream_handle):
        """Issue work on the cudaStream_t `stream_handle`; None = the context's own stream."""
        check(self._lib.mesh_ctx_set_stream(self.handle, ctypes.c_void_p(stream_handle or 0)), self.handle)

    def follow_torch(self, device):
        """Issue work on torch's current stream of `device`.  Torch's default
        stream has handle 0, which the C ABI reads as "the context's own
        stream"; it is passed as cudaStreamLegacy instead, so that the work is
        ordered after the kernels that produced the volume."""
        import torch
        h = torch.cuda.current_stream(device).cuda_stream
        self.set_stream(h if h else CUDA_STREAM_LEGACY)


def torch_dtype_code(dtype):
    """Volume dtype code of a torch dtype (None if unsupported)."""
    import torch
    return {torch.uint16: MESH_DT_U16, torch.float32: MESH_DT_F32, torch.float64: MESH_DT_F64,
            torch.int32: MESH_DT_I32, torch.int64: MESH_DT_I64, torch.float16: MESH_DT_F16, torch.int16: MESH_DT_I16,
            torch.int8: MESH_DT_I8, torch.uint8: MESH_DT_U8}.get(dtype)
