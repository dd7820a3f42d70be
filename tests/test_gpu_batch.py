"""Batched Marching Cubes (mesh_batch_*): many volumes in one pass.

Every volume of a batch must give exactly what isosurface() gives on that
volume alone -- the same vertices bit for bit, the same faces (1-based within
the volume), in the same order -- whatever the brick depth, CTA counts, scan
width or graph replay; a few volumes are also checked against the oracle.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def ragged(torch, n, seed, lo, hi, dtype):
    import meshing_gb300.fields as fields
    return fields.batch_volumes(n, seed=seed, lo=lo, hi=hi, dtype=dtype)


def check_alone(torch, pkg, b, vols, method, ranges=None, every=1):
    out = b.outputs()
    offs = out[2].cpu().numpy()
    assert offs[-1].tolist() == [b.nverts, b.nfaces]
    for i in range(0, len(vols), every):
        r = ranges[i] if ranges else ((-1, 1),) * 3
        v1, f1 = pkg.isosurface(vols[i], method, *r)
        v2, f2 = b.volume(i, out, offs)
        assert torch.equal(f1, f2), i
        assert torch.equal(v1, v2), i
    return out


def test_batch_matches_each_volume_alone(pkg, oracle, cuda):
    torch = cuda
    vols = ragged(torch, 60, 1, 2, 48, torch.float32)
    # volumes without cells (a side of 1) and the smallest with cells
    vols[3] = torch.zeros((1, 9, 9), device='cuda').permute(2, 1, 0).contiguous().permute(2, 1, 0)
    vols[7] = torch.tensor([[[-1.0, 1.0], [1.0, 1.0]], [[1.0, 1.0], [1.0, 1.0]]], device='cuda')
    m = pkg.MarchingCubes(iso=np.float32(0))
    b = pkg.Batch(vols, m)
    nv, nf = b.count()
    b.run()
    b.sync()
    check_alone(torch, pkg, b, vols, m)
    for i in (0, 5, 7, 59):
        A = np.asfortranarray(vols[i].cpu().numpy())
        want = oracle.isosurface(A, 'mc', np.float32(0), 1e-3, ((-1, 1),) * 3)
        v, f = b.volume(i)
        assert_same((v.cpu().numpy(), f.cpu().numpy()), want, str(i))
    assert nv > 1000 and nf > 500
    b.close()


def test_knobs_graph_and_tuner_keep_results(pkg, cuda):
    torch = cuda
    vols = ragged(torch, 40, 2, 16, 80, torch.float32)
    m = pkg.MarchingCubes(iso=np.float32(0))
    b = pkg.Batch(vols, m)
    b.count()
    b.run()
    b.sync()
    v0, f0, o0 = (t.clone() for t in b.outputs())
    for knobs in [dict(zs=16, classify_ctas=1, compact_ctas=2, scan_threads=256),
                  dict(zs=8, classify_ctas=2, compact_ctas=1, scan_threads=96),
                  dict(zs=0, classify_ctas=0, compact_ctas=0, scan_threads=1024)]:
        b.set_knobs(**knobs)
        b.count()
        for graph in (False, True, True):
            b.set_graph(graph)
            b.run()
            b.sync()
            v, f, o = b.outputs()
            assert torch.equal(o, o0) and torch.equal(f, f0) and torch.equal(v, v0), (knobs, graph)
    rep = b.tune(reps=2)
    assert 'best' in rep
    b.run()
    b.sync()
    v, f, o = b.outputs()
    assert torch.equal(o, o0) and torch.equal(f, f0) and torch.equal(v, v0)
    b.close()


@pytest.mark.parametrize('dt', ['f64', 'u16', 'f16', 'i16', 'u8'])
def test_batch_dtypes_and_per_volume_ranges(pkg, cuda, dt):
    torch = cuda
    rng = np.random.default_rng(5)
    shapes = [tuple(int(s) for s in rng.integers(3, 40, 3)) for _ in range(25)]
    if dt == 'u16':
        vols = [(torch.rand(sh, device='cuda') * 1000).to(torch.int32).to(torch.uint16) for sh in shapes]
        m = pkg.MarchingCubes(iso=500)
    elif dt == 'i16':
        vols = [(torch.rand(sh, device='cuda') * 2000 - 1000).to(torch.int16) for sh in shapes]
        m = pkg.MarchingCubes(iso=7)
    elif dt == 'u8':
        vols = [(torch.rand(sh, device='cuda') * 255).to(torch.uint8) for sh in shapes]
        m = pkg.MarchingCubes(iso=np.float32(99.5))
    elif dt == 'f16':
        vols = ragged(torch, 25, 3, 3, 40, torch.float16)
        m = pkg.MarchingCubes(iso=np.float32(0.01))
    else:
        vols = ragged(torch, 25, 3, 3, 40, torch.float64)
        m = pkg.MarchingCubes(iso=0.01)
    ranges = [((float(a), float(a) + 2.0), (-1.0, float(c)), (0.5, 3.0)) for a, c in rng.uniform(-2, 2, (25, 2))]
    b = pkg.Batch(vols, m, ranges=ranges)
    b.count()
    b.set_graph(True)
    b.run()
    b.sync()
    check_alone(torch, pkg, b, vols, m, ranges)
    b.close()


def test_outputs_larger_than_counted_are_reported(pkg, cuda):
    torch = cuda
    vols = ragged(torch, 12, 4, 16, 40, torch.float32)
    m = pkg.MarchingCubes(iso=np.float32(0))
    b = pkg.Batch(vols, m)
    b.count()
    vols[5].copy_(torch.rand_like(vols[5]) - 0.5)  # far more surface than counted
    b.run()
    with pytest.raises(pkg.MeshError) as ei:
        b.sync()
    assert ei.value.status == 6  # MESH_ECAPACITY
    b.count()
    b.run()
    b.sync()
    check_alone(torch, pkg, b, vols, m)
    b.close()


def test_uneven_batch_of_512(pkg, cuda):
    # the batched workload's shapes (16..128 per axis), 512 volumes
    torch = cuda
    vols = ragged(torch, 512, 0, 16, 128, torch.float32)
    m = pkg.MarchingCubes(iso=np.float32(0))
    b = pkg.Batch(vols, m)
    b.tune(reps=1)
    b.set_graph(True)
    b.run()
    b.sync()
    check_alone(torch, pkg, b, vols, m, every=7)
    b.close()


@pytest.mark.parametrize('dt', ['f32', 'f64', 'u16'])
def test_welded_batch_matches_each_volume_alone(pkg, oracle, cuda, dt):
    # MarchingCubes(weld=True) over a batch: each volume's welded mesh (its own
    # rows of the welded offsets, faces 1-based within it) equals the welded
    # isosurface() of the volume alone -- one run after the count, graph replays,
    # and a run on changed contents with fewer crossings
    torch = cuda
    rng = np.random.default_rng(9)
    ranges = None
    if dt == 'u16':
        shapes = [tuple(int(s) for s in rng.integers(3, 36, 3)) for _ in range(30)]
        vols = [(torch.rand(sh, device='cuda') * 1000).to(torch.int32).to(torch.uint16) for sh in shapes]
        m = pkg.MarchingCubes(iso=500, weld=True)
        ranges = [((float(a), float(a) + 2.0), (-1.0, float(c)), (0.5, 3.0)) for a, c in rng.uniform(-2, 2, (30, 2))]
    else:
        vols = ragged(torch, 40, 7, 2, 44, torch.float32 if dt == 'f32' else torch.float64)
        vols[3] = torch.zeros((1, 9, 9), device='cuda', dtype=vols[0].dtype)  # no cells
        vols[11] = torch.ones((6, 5, 7), device='cuda', dtype=vols[0].dtype)   # cells, no crossings
        m = pkg.MarchingCubes(iso=np.float32(0) if dt == 'f32' else 0.0, weld=True)
    b = pkg.Batch(vols, m, ranges=ranges)
    nv, nf = b.count()
    check_alone(torch, pkg, b, vols, m, ranges)  # the count's own run
    b.set_graph(True)
    for _ in range(2):
        b.run()
        b.sync()
    check_alone(torch, pkg, b, vols, m, ranges)
    if dt != 'u16':
        for i in (0, 5, 39):
            A = np.asfortranarray(vols[i].cpu().numpy())
            want = oracle.isosurface(A, 'mcw', m.iso, 1e-3, ((-1, 1),) * 3)
            v, f = b.volume(i)
            assert_same((v.cpu().numpy(), f.cpu().numpy()), want, 'welded batch volume %d' % i)
        # the per-cell batch of the same volumes: same faces, more vertices
        c = pkg.Batch(vols, pkg.MarchingCubes(iso=m.iso))
        nv_cell, nf_cell = c.count()
        assert nf_cell == nf and nv < nv_cell
        c.close()
        # fewer crossings after the count: a run reports the new welded rows
        vols[5].copy_(torch.full_like(vols[5], 1.0))
        b.run()
        b.sync()
        offs = b.outputs()[2].cpu().numpy()
        v5 = offs[6] - offs[5]
        assert v5.tolist() == [0, 0]
        b.nverts, b.nfaces = (int(x) for x in offs[-1])
        check_alone(torch, pkg, b, vols, m, ranges)
    b.close()
