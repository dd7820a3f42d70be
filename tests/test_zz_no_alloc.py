"""mesh_extract_noalloc: extraction for callers that cannot allocate.

Callbacks of a framework that owns the whole device memory pool, and
real-time loops that must never block in an allocator, cannot call cudaMalloc
when they extract a mesh.  mesh_extract_noalloc keeps its scratch in a static
device array of MESH_NOALLOC_SCRATCH_BYTES instead.  These tests call it
through the C ABI and check that it returns exactly what the allocating entry
point mesh_extract_device returns (the same contract as every parity test:
connectivity and counts bit-exact, positions within 1e-12 / 2 ulp -- here
bit-identical), on calls made back to back so that the second call runs on
the scratch the first one left behind, and, per algorithm, exactly the
oracle's mesh.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _volume(torch, shape, kind, dtype):
    g = [torch.linspace(-1, 1, n, dtype=torch.float64, device='cuda') for n in shape]
    x, y, z = g[0][:, None, None], g[1][None, :, None], g[2][None, None, :]
    if kind == 'sphere':
        f = torch.sqrt(x * x + y * y + z * z) - 0.55
    else:
        f = torch.sin(4 * x) * torch.cos(4 * y) + torch.sin(4 * y) * torch.cos(4 * z) + torch.sin(4 * z) * torch.cos(4 * x)
    # Julia layout: x fastest in memory
    return f.to(dtype).permute(2, 1, 0).contiguous().permute(2, 1, 0)


def _run_both(pkg, torch, vol, method, ranges):
    lib = pkg.load_library()
    p = pkg.make_params(method, *ranges)
    dt = pkg._lib.torch_dtype_code(vol.dtype)
    nx, ny, nz = vol.shape
    ref_counts = pkg.isosurface_device(vol, method, *ranges,
                                       verts=torch.empty((1, 3), device='cuda'),
                                       faces=torch.empty((1, 3), dtype=torch.int64, device='cuda'))
    try:
        pkg.api.sync()
    except pkg.MeshError:
        pass  # capacity 1: only the counts are wanted here
    nv, nf = ref_counts.tolist()
    npdt = {torch.float32: np.float32, torch.float64: np.float64, torch.int32: np.int32, torch.int64: np.int64,
            torch.uint16: np.uint16}[vol.dtype]
    bits = pkg.output_float_bits(npdt, method, *ranges)
    ft = torch.float32 if bits == 32 else torch.float64
    rv = torch.empty((nv, 3), dtype=ft, device='cuda')
    rf = torch.empty((nf, 3), dtype=torch.int64, device='cuda')
    c = pkg.isosurface_device(vol, method, *ranges, verts=rv, faces=rf)
    pkg.api.sync()
    assert c.tolist() == [nv, nf]

    nv_ = torch.full((nv + 7, 3), float('nan'), dtype=ft, device='cuda')
    nf_ = torch.full((nf + 5, 3), -7, dtype=torch.int64, device='cuda')
    counts = torch.full((3,), -1, dtype=torch.int64, device='cuda')
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.mesh_extract_noalloc(ctypes.c_void_p(vol.data_ptr()), dt, nx, ny, nz, ctypes.byref(p),
                                  ctypes.c_void_p(nv_.data_ptr()), nv + 7, ctypes.c_void_p(nf_.data_ptr()), nf + 5,
                                  ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, pkg._lib.STATUS.get(rc, rc)
    torch.cuda.synchronize()
    assert counts.tolist() == [nv, nf, 0]
    # bit-identical to the allocating path; nothing written past the mesh
    assert torch.equal(nf_[:nf], rf)
    assert torch.equal(nv_[:nv].view(torch.int32 if ft == torch.float32 else torch.int64),
                       rv.view(torch.int32 if ft == torch.float32 else torch.int64))
    assert bool(torch.isnan(nv_[nv:]).all()) and bool((nf_[nf:] == -7).all())
    return nv, nf


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(pkg, cuda):
    torch = cuda
    calls = [
        (_volume(torch, (120, 97, 133), 'waves', torch.float32), pkg.MarchingCubes(iso=np.float32(0.1)), ((0, 1),) * 3),
        (_volume(torch, (64, 64, 64), 'sphere', torch.float64), pkg.MarchingCubes(), ((-1, 1),) * 3),
        (_volume(torch, (41, 55, 38), 'waves', torch.float32), pkg.MarchingTetrahedra(iso=np.float32(0)),
         ((0, 1),) * 3),
        (_volume(torch, (50, 47, 61), 'sphere', torch.float32), pkg.NaiveSurfaceNets(iso=np.float32(0)),
         ((-1, 1),) * 3),
    ]
    sizes = [_run_both(pkg, torch, *c) for c in calls]
    assert all(nv > 0 and nf > 0 for nv, nf in sizes)
    # the same call twice in a row gives the same answer
    assert _run_both(pkg, torch, *calls[0]) == sizes[0]


def test_noalloc_integer_and_uint16_volumes(pkg, cuda):
    # the integer-vs-iso thresholds and Int / Int quotients of the context path
    torch = cuda
    base = _volume(torch, (47, 52, 45), 'sphere', torch.float64)
    i32 = (base * 1000).round().to(torch.int32)
    i64 = (base * 3e15).round().to(torch.int64)
    u = np.round((base.cpu().numpy() + 1) * 20000).astype(np.uint16)  # Julia layout, as base
    u16 = torch.from_numpy(np.ascontiguousarray(u.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
    calls = [
        (i32, pkg.MarchingCubes(iso=7), ((-1, 1),) * 3),
        (i64, pkg.MarchingCubes(iso=12345), ((0, 1),) * 3),
        (i32, pkg.MarchingTetrahedra(iso=-3), ((-1, 1),) * 3),
        (u16, pkg.MarchingCubes(iso=20500), ((-1, 1),) * 3),
        (u16, pkg.NaiveSurfaceNets(iso=np.float32(20000.5)), ((-1, 1),) * 3),
    ]
    for c in calls:
        nv, nf = _run_both(pkg, torch, *c)
        assert nv > 0 and nf > 0


def test_noalloc_rejects_calls_beyond_its_scratch(pkg, cuda):
    torch = cuda
    lib = pkg.load_library()
    vol = _volume(torch, (32, 32, 32), 'sphere', torch.float32)
    p = pkg.make_params(pkg.MarchingCubes(iso=np.float32(0)), (-1, 1), (-1, 1), (-1, 1))
    counts = torch.zeros(3, dtype=torch.int64, device='cuda')
    dummy = torch.empty((1, 3), dtype=torch.float32, device='cuda')
    # room for 2^31 vertices would need ~2^29 active-cell entries: far beyond 64 MiB
    rc = lib.mesh_extract_noalloc(ctypes.c_void_p(vol.data_ptr()), 2, 32, 32, 32, ctypes.byref(p),
                                  ctypes.c_void_p(dummy.data_ptr()), 1 << 31, ctypes.c_void_p(dummy.data_ptr()), 1,
                                  ctypes.c_void_p(counts.data_ptr()), None)
    assert rc == 8  # MESH_ESCRATCH
    assert lib.mesh_status_string(8) == b'needs more scratch than the no-allocation limit'


@pytest.mark.parametrize('alg', ['mc', 'mt', 'nsn'])
def test_noalloc_matches_the_oracle(pkg, oracle, cuda, alg):
    # one whole z segment per column (the tiling this entry point uses) against
    # the CPU oracle, bit for bit
    torch = cuda
    vol = _volume(torch, (45, 38, 70), 'waves', torch.float32)
    A = np.asfortranarray(vol.cpu().numpy())
    iso, ranges = np.float32(0.05), ((0.0, 1.0), (-1.0, 1.0), (0.0, 2.0))
    method = {'mc': pkg.MarchingCubes(iso=iso), 'mt': pkg.MarchingTetrahedra(iso=iso, eps=1e-3),
              'nsn': pkg.NaiveSurfaceNets(iso=iso)}[alg]
    wv, wf = oracle.isosurface(A, alg, iso, 1e-3, ranges)
    ft = torch.float32 if wv.dtype == np.float32 else torch.float64
    verts = torch.empty((len(wv), 3), dtype=ft, device='cuda')
    faces = torch.empty((len(wf), 3), dtype=torch.int64, device='cuda')
    counts = torch.full((3,), -1, dtype=torch.int64, device='cuda')
    p = pkg.make_params(method, *ranges)
    lib = pkg.load_library()
    for _ in range(2):  # twice in a row on the same scratch
        rc = lib.mesh_extract_noalloc(ctypes.c_void_p(vol.data_ptr()), 2, *vol.shape, ctypes.byref(p),
                                      ctypes.c_void_p(verts.data_ptr()), len(wv), ctypes.c_void_p(faces.data_ptr()),
                                      len(wf), ctypes.c_void_p(counts.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        assert counts.tolist() == [len(wv), len(wf), 0]
        assert np.array_equal(faces.cpu().numpy(), wf)
        assert np.array_equal(verts.cpu().numpy().view(np.uint8), wv.view(np.uint8))
