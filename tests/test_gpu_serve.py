"""Serving loop (mesh_server_*): continuous batching of mixed requests.

Every request must give exactly the mesh isosurface() gives for it alone,
whether it ran alone or in a wave with others (Marching Cubes requests of a
wave share one batch; waves overlap on the device), from a device or a host
volume, welded or not; admission respects the memory budget and the queue
limit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALG = ('MarchingCubes', 'MarchingTetrahedra', 'NaiveSurfaceNets')


def requests(torch, pkg, n, seed, lo=6, hi=90):
    import meshing_gb300.fields as fields
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        shape = tuple(int(s) for s in rng.integers(lo, hi, 3))
        dt = torch.float32 if rng.random() < 0.5 else torch.float64
        if rng.random() < 0.5:
            A = fields.primitives_sdf(shape, fields.primitives_params(rng), dtype=dt)
        else:
            A = (torch.rand(shape, device='cuda', dtype=torch.float64) - 0.5).to(dt)
        a = rng.choice(3, p=[0.6, 0.3, 0.1])
        iso = np.float32(0) if dt == torch.float32 and rng.random() < 0.7 else 0.0
        m = pkg.MarchingTetrahedra(iso=iso) if a == 1 else getattr(pkg, ALG[a])(iso=iso)
        r = ((-1, 1), (-1, 1), (-1, 1)) if rng.random() < 0.7 else ((0.0, 2.0), (-1.5, 1.0), (0.0, 0.5))
        out.append((A, m, r))
    return out


def same(torch, got, want):
    return torch.equal(got[1], want[1]) and torch.equal(got[0], want[0])


def test_mix_equals_alone_equals_isosurface(pkg, cuda):
    torch = cuda
    reqs = requests(torch, pkg, 48, 1)
    want = [pkg.isosurface(A, m, *r) for A, m, r in reqs]
    srv = pkg.Server(budget_bytes=6 << 30, slots=2, max_wave=16)
    # in the mix: everything queued at once, answered in overlapping waves
    ids = [srv.submit(A, m, *r) for A, m, r in reqs]
    for i, rid in enumerate(ids):
        got = srv.result(rid)
        assert same(torch, got, want[i]), i
        srv.release(rid)
    st = srv.stats()
    assert st['completed'] == len(reqs) and st['failed'] == 0 and st['rejected'] == 0
    assert st['peak_reserved_bytes'] <= st['pool_bytes']
    # alone: one request in flight at a time
    for i, (A, m, r) in enumerate(reqs[:12]):
        rid = srv.submit(A, m, *r)
        assert same(torch, srv.result(rid), want[i]), i
        srv.release(rid)
    srv.close()


def test_admission_waits_for_memory_and_limits_the_queue(pkg, cuda):
    torch = cuda
    gen = torch.Generator(device='cuda').manual_seed(3)
    dense = torch.rand((100, 100, 100), device='cuda', generator=gen)  # nearly every cell active
    m = pkg.MarchingCubes(iso=np.float32(0.5))
    want = pkg.isosurface(dense, m)
    # W: what one request reserves in flight (worst case); K: what its finished mesh keeps
    probe = pkg.Server(budget_bytes=4 << 30)
    rid = probe.submit(dense, m)
    probe.wait(rid)
    st = probe.stats()
    W, K = int(st['peak_reserved_bytes']), int(st['reserved_bytes'])
    probe.close()
    assert 0 < K < W
    # room for one request in flight, but not beside a finished, unreleased mesh
    srv = pkg.Server(budget_bytes=W + K // 2, slots=2, max_wave=4, max_queue=2)
    a = srv.submit(dense, m)
    assert same(torch, srv.result(a), want)   # done, its mesh still reserved
    b = srv.submit(dense, m)
    c = srv.submit(dense, m)
    with pytest.raises(pkg.MeshError) as ei:
        srv.submit(dense, m)                    # two waiting: queue full
    assert ei.value.status == 10  # MESH_EBUSY
    assert srv.poll(b) == 'queued'              # no memory until a is released
    srv.release(a)
    for rid in (b, c):                          # one at a time, each after the previous release
        assert same(torch, srv.result(rid), want)
        srv.release(rid)
    # a worst case beyond the whole budget is rejected at once
    huge = torch.rand((160, 160, 160), device='cuda', generator=gen)
    with pytest.raises(pkg.MeshError) as ei:
        srv.submit(huge, m)
    assert ei.value.status == 9  # MESH_EBUDGET
    st = srv.stats()
    assert st['rejected'] == 2 and st['completed'] == 3 and st['peak_reserved_bytes'] <= st['pool_bytes']
    srv.close()


def test_empty_and_degenerate_requests(pkg, cuda):
    torch = cuda
    srv = pkg.Server(budget_bytes=256 << 20)
    cases = [torch.ones((5, 6, 7), device='cuda'), torch.zeros((1, 8, 8), device='cuda'),
             -torch.ones((9, 9, 9), device='cuda', dtype=torch.float64)]
    for A in cases:
        for m in (pkg.MarchingCubes(), pkg.MarchingTetrahedra(), pkg.NaiveSurfaceNets()):
            rid = srv.submit(A, m)
            v, f = srv.result(rid)
            assert v.shape[0] == 0 and f.shape[0] == 0
            srv.release(rid)
    srv.close()


def test_bursts_and_concurrent_submitters(pkg, cuda):
    # many requests submitted at once and from several threads while waves are
    # being launched (the server's request map grows while waves are queued)
    torch = cuda
    import threading
    import meshing_gb300.fields as fields
    rng = np.random.default_rng(21)
    vols = [fields.primitives_sdf((48, 40, 56), fields.primitives_params(rng)) for _ in range(8)]
    m = pkg.MarchingCubes(iso=np.float32(0))
    want = [pkg.isosurface(v, m) for v in vols]
    srv = pkg.Server(budget_bytes=8 << 30, slots=3, max_wave=64)
    srv.replay([(vols[i % 8], m, ((-1, 1),) * 3) for i in range(512)], np.zeros(512))
    st = srv.stats()
    assert st['completed'] == 512 and st['failed'] == 0
    ids = [[] for _ in range(4)]

    def submit(k):
        for i in range(120):
            ids[k].append((i % 8, srv.submit(vols[i % 8], m)))

    th = [threading.Thread(target=submit, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for lst in ids:
        for i, rid in lst:
            assert same(torch, srv.result(rid), want[i])
            srv.release(rid)
    srv.close()


def test_small_int_and_float16_requests(pkg, cuda):
    # Float16 / Int16 / UInt8 / Int8 volumes through the serving loop, every algorithm,
    # equal to the volume's own isosurface call; welded meshes are not served
    torch = cuda
    rng = np.random.default_rng(9)
    vols = [
        (torch.rand((21, 30, 17), device='cuda').to(torch.float16), np.float32(0.5)),
        ((torch.rand((25, 19, 33), device='cuda') * 2000 - 1000).to(torch.int16), 0),
        ((torch.rand((18, 27, 22), device='cuda') * 255).to(torch.uint8), 128),
        ((torch.rand((23, 23, 23), device='cuda') * 250 - 125).to(torch.int8), np.float32(0.5)),
    ]
    srv = pkg.Server(budget_bytes=2 << 30)
    for A, iso in vols:
        for m in (pkg.MarchingCubes(iso=iso), pkg.MarchingTetrahedra(iso=iso, eps=np.float32(1e-3)),
                  pkg.NaiveSurfaceNets(iso=iso), pkg.MarchingCubes(iso=iso, weld=True)):
            want = pkg.isosurface(A, m)
            rid = srv.submit(A, m)
            assert same(torch, srv.result(rid), want), (A.dtype, type(m).__name__)
            srv.release(rid)
    srv.close()
    del rng


def test_host_volumes_and_welded_requests_alone_and_in_the_mix(pkg, cuda):
    # requests whose volumes are host arrays (uploaded into the pool at
    # admission) and welded Marching Cubes requests, mixed with device
    # requests: every result equals the request's own isosurface call, in the
    # mix and alone, and the host volumes' pool blocks are returned
    torch = cuda
    reqs = requests(torch, pkg, 40, 5)
    mixed = []
    for i, (A, m, r) in enumerate(reqs):
        if i % 3 == 0:
            A = A.cpu().numpy()                           # host volume
        if i % 4 == 1 and type(m).__name__ == 'MarchingCubes':
            m = pkg.MarchingCubes(iso=m.iso, weld=True)   # welded
        mixed.append((A, m, r))
    want = [pkg.isosurface(torch.from_numpy(A).cuda() if isinstance(A, np.ndarray) else A, m, *r)
            for A, m, r in mixed]
    assert any(isinstance(A, np.ndarray) for A, _, _ in mixed) and any(getattr(m, 'weld', False) for _, m, _ in mixed)
    srv = pkg.Server(budget_bytes=6 << 30, slots=3, max_wave=16)
    ids = [srv.submit(A, m, *r) for A, m, r in mixed]
    for i, rid in enumerate(ids):
        got = srv.result(rid)
        assert same(torch, got, want[i]), i
        srv.release(rid)
    st = srv.stats()
    assert st['completed'] == len(mixed) and st['failed'] == 0
    assert st['reserved_bytes'] == 0                      # host volumes' copies given back
    for i, (A, m, r) in enumerate(mixed[:9]):
        rid = srv.submit(A, m, *r)
        assert same(torch, srv.result(rid), want[i]), i
        srv.release(rid)
    srv.close()


def test_host_volume_bytes_count_against_the_budget(pkg, cuda):
    # a host request's worst case includes its volume's pool copy: a budget that
    # holds the outputs of a device request but not the volume beside them
    # rejects the same request from host memory
    torch = cuda
    A = torch.rand((64, 64, 64), device='cuda', dtype=torch.float64)
    m = pkg.NaiveSurfaceNets(iso=0.5)
    probe = pkg.Server(budget_bytes=1 << 30)
    rid = probe.submit(A, m)
    probe.wait(rid)
    W = int(probe.stats()['peak_reserved_bytes'])   # outputs of the device request
    probe.close()
    srv = pkg.Server(budget_bytes=W + (64 ** 3 * 8) // 2)
    rid = srv.submit(A, m)
    srv.result(rid)
    srv.release(rid)
    with pytest.raises(pkg.MeshError) as ei:
        srv.submit(A.cpu().numpy(), m)
    assert ei.value.status == 9  # MESH_EBUDGET
    srv.close()
