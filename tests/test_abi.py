"""C ABI and host logic checks that need no GPU: the library loads, exports
every symbol the header declares, and its host-side type planning and argument
validation behave like the reference's type rules."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'meshing_gb300.h')).read()
    return sorted(set(re.findall(r'MESH_API\s+[\w\s\*]*?\b(mesh_\w+)\s*\(', src)))


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg._lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) == 36
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(pkg._lib.EXPORTS) == names


def test_params_default_mirror_reference(pkg):
    p = pkg.MeshParams()
    pkg.load_library().mesh_params_default(ctypes.byref(p))
    assert (p.alg, p.iso_type, p.iso, p.eps_type, p.eps, p.range_type) == (0, 3, 0.0, 3, 1e-3, 4)
    assert list(p.range) == [-1, 1, -1, 1, -1, 1]


@pytest.mark.parametrize('dtype,method,rng,bits', [
    (np.float64, ('mc', 0.0), (-1, 1), 64),
    (np.float32, ('mc', 0.0), (-1, 1), 64),
    (np.float32, ('mc', np.float32(0)), (-1, 1), 32),
    (np.float32, ('mc', 0), (-1, 1), 32),
    (np.float32, ('mc', np.float32(0)), (-1.0, 1.0), 64),
    (np.float32, ('mc', np.float32(0)), (np.float32(-1), np.float32(1)), 32),
    (np.uint16, ('mc', 500), (-1, 1), 64),
    (np.uint16, ('mc', np.float32(500)), (-1, 1), 32),
    (np.float32, ('mt', np.float32(0), np.float32(1e-3)), (-1, 1), 32),
    (np.float32, ('mt', np.float32(0), 1e-3), (-1, 1), 64),
    (np.float32, ('nsn', np.float32(0)), (-1, 1), 32),
    (np.float16, ('mc', 0.0), (-1, 1), 64),
    (np.float16, ('mc', np.float32(0)), (-1, 1), 32),
    (np.float16, ('mc', np.float32(0)), (-1.0, 1.0), 64),
    (np.float16, ('mt', np.float32(0), np.float32(1e-3)), (np.float32(0), np.float32(1)), 32),
])
def test_output_eltype_matches_oracle(pkg, oracle, dtype, method, rng, bits):
    alg = method[0]
    m = {'mc': pkg.MarchingCubes, 'nsn': pkg.NaiveSurfaceNets}.get(alg)
    meth = pkg.MarchingTetrahedra(iso=method[1], eps=method[2]) if alg == 'mt' else m(iso=method[1])
    assert pkg.output_float_bits(dtype, meth, rng, rng, rng) == bits
    rt = {int: 4, float: 3, np.float32: 2}[type(rng[0])]
    eps = method[2] if alg == 'mt' else 1e-3
    assert oracle.output_bits(dtype, alg, method[1], eps, rt) == bits


def test_invalid_arguments_rejected(pkg):
    with pytest.raises(TypeError):
        pkg.make_params(pkg.MarchingCubes(iso=True))
    with pytest.raises(TypeError):
        pkg.make_params(pkg.MarchingCubes(), (-1, 1.0), (-1, 1), (-1, 1))  # mixed endpoint types
    with pytest.raises(TypeError):
        pkg.make_params(pkg.MarchingTetrahedra(eps=0))
    p = pkg.make_params(pkg.MarchingCubes())
    p.range[0] = float('inf')
    bits = ctypes.c_int()
    rc = pkg.load_library().mesh_output_float_bits(2, ctypes.byref(p), ctypes.byref(bits))
    assert rc == 1  # MESH_EINVAL
    p = pkg.make_params(pkg.MarchingCubes(iso=np.float32(0)))
    p.iso = 0.1  # not a Float32 value
    assert pkg.load_library().mesh_output_float_bits(2, ctypes.byref(p), ctypes.byref(bits)) == 1
    assert pkg.load_library().mesh_output_float_bits(9, ctypes.byref(p), ctypes.byref(bits)) == 1
    # Float16 data with an Int iso would divide in Float16 arithmetic: not taken
    p = pkg.make_params(pkg.MarchingCubes(iso=0))
    assert pkg.load_library().mesh_output_float_bits(6, ctypes.byref(p), ctypes.byref(bits)) == 1
    p = pkg.make_params(pkg.MarchingCubes(iso=np.float32(0)))
    assert pkg.load_library().mesh_output_float_bits(6, ctypes.byref(p), ctypes.byref(bits)) == 0


def test_generic_forwarder_defaults_to_marching_cubes(pkg):
    # isosurface(A, args...) = isosurface(A, MarchingCubes(), args...)  (src/isosurface.jl:30-32)
    m, rest = pkg.api._split_args(((0, 1), (0, 1), (0, 1)))
    assert m == pkg.MarchingCubes() and len(rest) == 3
    m, rest = pkg.api._split_args((pkg.MarchingTetrahedra(iso=0.5),))
    assert m == pkg.MarchingTetrahedra(iso=0.5) and rest == ()


def test_range_arguments(pkg):
    # first(X) / last(X) of ranges, sequences and (first, last) pairs
    p = pkg.make_params(pkg.MarchingCubes(), range(-2, 3), [0, 5, 1], (-1, 1))
    assert list(p.range) == [-2, 2, 0, 1, -1, 1] and p.range_type == 4
    p = pkg.make_params(pkg.MarchingCubes(), np.array([0.0, 0.5, 1.0]), (np.float64(-1), 1.0), (0.0, 2.0))
    assert list(p.range) == [0, 1, -1, 1, 0, 2] and p.range_type == 3


def test_torch_default_stream_is_passed_as_the_legacy_stream(pkg, monkeypatch):
    # torch's default stream has handle 0, which mesh_ctx_set_stream reads as
    # "the context's own (non-blocking) stream"; work on a torch volume must be
    # ordered after the kernels that wrote it, so the binding passes
    # cudaStreamLegacy (1) instead, and other streams unchanged
    import torch
    from meshing_gb300 import _lib

    seen = []

    class FakeLib:
        def mesh_ctx_set_stream(self, h, s):
            seen.append(s.value)
            return 0

        def mesh_ctx_destroy(self, h):
            pass

    class FakeStream:
        def __init__(self, h):
            self.cuda_stream = h

    c = _lib.Context.__new__(_lib.Context)
    c._lib, c.handle, c.device = FakeLib(), ctypes.c_void_p(1234), 0
    for h, want in [(0, 1), (0xabc000, 0xabc000)]:
        monkeypatch.setattr(torch.cuda, 'current_stream', lambda device=None, h=h: FakeStream(h))
        c.follow_torch(0)
        assert seen[-1] == want
    c.set_stream(None)
    assert seen[-1] is None  # NULL: the context's own stream
    c.handle = None
