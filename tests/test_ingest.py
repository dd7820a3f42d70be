"""Volume ingest (meshing.jl_gb300/ingest.py): NRRD and raw files, the path of
the reference's CT example (examples/nrrd.jl: load an NRRD volume, mesh it with
iso 100)."""
import gzip
import os

import numpy as np
import pytest


@pytest.fixture(scope='module')
def ingest(pkg):
    import meshing_gb300.ingest as ing
    return ing


DTYPES = [np.int16, np.uint8, np.int8, np.uint16, np.int32, np.int64, np.float32, np.float64]


@pytest.mark.parametrize('dt', DTYPES)
def test_nrrd_round_trip_every_encoding(ingest, tmp_path, dt):
    rng = np.random.default_rng(np.dtype(dt).itemsize)
    A = np.asfortranarray((rng.standard_normal((9, 6, 5)) * 90).astype(dt))
    for enc in ('raw', 'gzip', 'bzip2', 'ascii'):
        for detached in (False, True):
            for endian in ('little', 'big'):
                p = str(tmp_path / ('v_%s_%d_%s.nrrd' % (enc, detached, endian)))
                ingest.write_nrrd(p, A, encoding=enc, detached=detached, endian=endian)
                B, hdr = ingest.read_nrrd(p)
                assert hdr['shape'] == (9, 6, 5)
                assert B.dtype == A.dtype and B.flags.f_contiguous and np.array_equal(A, B), (enc, detached, endian)


def test_nrrd_header_geometry_and_skips(ingest, tmp_path):
    A = np.asfortranarray(np.arange(4 * 3 * 2, dtype=np.int16).reshape((4, 3, 2), order='F'))
    p = str(tmp_path / 'g.nrrd')
    ingest.write_nrrd(p, A, spacing=(0.5, 0.25, 2.0), origin=(1.0, -2.0, 3.0))
    B, hdr = ingest.read_nrrd(p)
    assert np.array_equal(A, B)
    assert hdr['ranges'] == ((1.0, 2.5), (-2.0, -1.5), (3.0, 5.0))
    # byte skip / line skip, a leading size-1 axis, comments and key/value pairs
    body = A.transpose(2, 1, 0).astype('<i2').tobytes()
    q = tmp_path / 's.nrrd'
    q.write_bytes(b'NRRD0005\n# a comment\ntype: short\ndimension: 4\nsizes: 1 4 3 2\nendian: little\n'
                  b'encoding: raw\nbyte skip: 3\nline skip: 1\nmodality:=CT\n\nheader line\nXYZ' + body)
    C, h2 = ingest.read_nrrd(str(q))
    assert np.array_equal(A, C) and h2['keyvalue'] == {'modality': 'CT'}
    # byte skip -1: the data sits at the end of the (detached) file
    (tmp_path / 'tail.raw').write_bytes(b'junk' * 5 + gzip.decompress(gzip.compress(body)))
    (tmp_path / 't.nhdr').write_bytes(b'NRRD0004\ntype: int16\ndimension: 3\nsizes: 4 3 2\nendian: little\n'
                                      b'encoding: raw\nbyte skip: -1\ndata file: tail.raw\n')
    D, _ = ingest.read_nrrd(str(tmp_path / 't.nhdr'))
    assert np.array_equal(A, D)
    # axis mins / maxs give the ranges directly
    (tmp_path / 'm.nrrd').write_bytes(b'NRRD0004\ntype: uint8\ndimension: 3\nsizes: 2 2 2\nencoding: raw\n'
                                      b'axis mins: -1 -2 -3\naxis maxs: 1 2 3\n\n' + bytes(range(8)))
    E, h3 = ingest.read_nrrd(str(tmp_path / 'm.nrrd'))
    assert h3['ranges'] == ((-1.0, 1.0), (-2.0, 2.0), (-3.0, 3.0)) and E[1, 0, 0] == 1 and E[0, 0, 1] == 4


def test_nrrd_rejections(ingest, tmp_path):
    bad = [
        b'NRRD0004\ntype: uint32\ndimension: 3\nsizes: 2 2 2\nencoding: raw\n\n' + bytes(32),   # no kernel
        b'NRRD0004\ntype: float\ndimension: 2\nsizes: 2 2\nencoding: raw\n\n' + bytes(16),      # not 3-D
        b'NRRD0004\ntype: float\ndimension: 3\nsizes: 2 2 2\nencoding: raw\n\n' + bytes(16),    # too short
        b'NRRD0004\ntype: float\ndimension: 3\nsizes: 2 2 2\nencoding: hex\n\n' + bytes(64),    # encoding
        b'NRRD0004\ntype: float\ndimension: 3\nsizes: 2 2 2\nencoding: raw\ndata file: LIST\na\nb\n',
        b'P6\n2 2\n255\n',                                                                        # not NRRD
    ]
    for i, blob in enumerate(bad):
        p = tmp_path / ('bad%d.nrrd' % i)
        p.write_bytes(blob)
        with pytest.raises(ValueError):
            ingest.read_nrrd(str(p))


def test_raw_reader(ingest, tmp_path):
    A = np.asfortranarray(np.random.default_rng(3).integers(0, 4000, (6, 5, 4)).astype(np.uint16))
    p = tmp_path / 'v.raw'
    p.write_bytes(b'\0' * 10 + A.transpose(2, 1, 0).astype('>u2').tobytes())
    B = ingest.read_raw(str(p), (6, 5, 4), np.uint16, offset=10, endian='big')
    assert B.dtype == np.uint16 and np.array_equal(A, B)
    with pytest.raises(ValueError):
        ingest.read_raw(str(p), (7, 5, 4), np.uint16, offset=10, endian='big')


@pytest.mark.gpu
def test_nrrd_ct_volume_through_the_device(pkg, oracle, cuda, ingest, tmp_path):
    # examples/nrrd.jl: a CT volume of Int16 values meshed with iso 100 (an Int) by each
    # algorithm, with the default X = Y = Z = -1:1; here a seeded CT-like volume
    rng = np.random.default_rng(100)
    n = (41, 37, 45)
    g = [np.linspace(-1, 1, k) for k in n]
    X, Y, Z = np.meshgrid(*g, indexing='ij')
    shell = np.abs(np.sqrt(X ** 2 / 0.5 + Y ** 2 / 0.3 + Z ** 2 / 0.6) - 0.8) < 0.08
    A = np.clip(rng.normal(-50, 30, n) + shell * rng.normal(400, 40, n), -1024, 3071).astype(np.int16)
    p = str(tmp_path / 'ct.nrrd')
    ingest.write_nrrd(p, np.asfortranarray(A), encoding='gzip', spacing=(0.7, 0.7, 1.25))
    V, hdr = ingest.read_nrrd(p, device='cuda')
    assert tuple(V.shape) == n and V.dtype == cuda.int16
    for alg, m in (('mc', pkg.MarchingCubes(iso=100)), ('mt', pkg.MarchingTetrahedra(iso=100)),
                   ('nsn', pkg.NaiveSurfaceNets(iso=100))):
        v, f = pkg.isosurface(V, m)
        cuda.cuda.synchronize()
        wv, wf = oracle.isosurface(np.asfortranarray(A), alg, 100, 1e-3)
        assert v.dtype == cuda.float64 and len(wf) > 0
        assert np.array_equal(f.cpu().numpy(), wf) and np.array_equal(v.cpu().numpy(), wv), alg
