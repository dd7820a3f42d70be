#!/usr/bin/env python3
"""Generate ``mesh_tables.h``: the per-case lookup tables the CUDA kernels use.

The tables are *derived* from Meshing.jl v0.7.0's lookup tables, which the GPU
path must reproduce bit-for-bit (case selection, vertex order and face
connectivity are part of the output contract):

* Marching Cubes: ``_mc_verts`` (src/lut/mc.jl:301-555), ``_mc_eq_mapping``
  (src/lut/mc.jl:557-579), ``_mc_connectivity`` (src/lut/mc.jl:581-604) and
  ``_mc_edge_list`` (src/lut/mc.jl:606-608), used by ``process_mc_voxel!``
  (src/marching_cubes.jl:67-92).
* Marching Tetrahedra: ``voxCrnrPos``, ``voxEdgeCrnrs``, ``voxEdgeDir``,
  ``voxEdgeIx``, ``subTets``, ``subTetsMask``, ``tetEdgeCrnrs``, ``tetTri``
  (src/lut/mt.jl:23-107), used by ``tetIx``/``procVox``
  (src/marching_tetrahedra.jl:11-18,105-127).

Instead of the reference's nested tuples, every cube case (0..255) is flattened
into the exact emission sequence ``process_mc_voxel!`` / ``procVox`` produce
for it, packed for constant/shared memory.  Before writing, the script checks
the MC tables against the classic ``tri_table`` (src/lut/mc.jl:46-299), which
``src/`` does not use: vertex slots must be the crossed edges in first-use
order of ``tri_table[c]`` and each face must be a reversed ``tri_table``
triple.

Run by hand (it reads the reference checkout given as argv[1]); the output is
committed, so builds never need the reference.
"""
import os
import re
import sys


def _grab(src, name):
    i = src.index('const ' + name)
    j = src.find('\nconst', i + 1)
    body = src[i:j if j > 0 else len(src)]
    return '\n'.join(line.split('#')[0] for line in body.split('\n'))


def _rows(body):
    inner = body[body.index('(') + 1:]
    return [[int(x, 0) for x in r.replace(' ', '').replace('\n', '').split(',') if x]
            for r in re.findall(r'\(([^()]*)\)', inner)]


def _flat(body):
    return [int(x, 16) for x in re.findall(r'0x[0-9a-f]+', body)]


def load_mc(path):
    src = open(os.path.join(path, 'src/lut/mc.jl')).read()
    verts = _rows(_grab(src, '_mc_verts'))
    eqmap = _flat(_grab(src, '_mc_eq_mapping'))
    conn = _rows(_grab(src, '_mc_connectivity'))
    elist = _rows(_grab(src, '_mc_edge_list'))
    tri = _rows(_grab(src, 'tri_table'))
    assert len(verts) == 254 and len(eqmap) == 254 and len(conn) == 24
    assert len(elist) == 12 and len(tri) == 254
    return verts, eqmap, conn, elist, tri


def load_mt(path):
    src = open(os.path.join(path, 'src/lut/mt.jl')).read()
    out = {}
    for name in ('voxCrnrPos', 'voxEdgeCrnrs', 'voxEdgeIx', 'subTets', 'subTetsMask',
                 'tetEdgeCrnrs', 'tetTri'):
        out[name] = _rows(_grab(src, name))
    out['voxEdgeDir'] = _flat(_grab(src, 'voxEdgeDir'))
    return out


def mc_cases(verts, eqmap, conn):
    """Per case: (edge of each local vertex slot, faces as local-slot triples).

    Mirrors process_mc_voxel! (src/marching_cubes.jl:67-92): slots follow
    _mc_verts[c] up to the first zero; the first face is (3,2,1); further faces
    come from _mc_connectivity[_mc_eq_mapping[c]] in groups of three, reversed,
    until a zero entry.
    """
    cases = [([], [])]
    for c in range(1, 255):
        row = verts[c - 1]
        edges = []
        for v in row:
            if v == 0:
                break
            edges.append(v - 1)
        faces = [(2, 1, 0)]
        o = conn[eqmap[c - 1] - 1]
        for i in (0, 3, 6, 9):
            if o[i] == 0:
                break
            faces.append((o[i + 2] - 1, o[i + 1] - 1, o[i] - 1))
        cases.append((edges, faces))
    cases.append(([], []))
    return cases


def check_mc_against_tri_table(cases, tri):
    for c in range(1, 255):
        edges, faces = cases[c]
        seq = [e - 1 for e in tri[c - 1] if e != 0]
        assert len(seq) % 3 == 0
        first = []
        for e in seq:
            if e not in first:
                first.append(e)
        assert first == edges, ('vertex order', c)
        slot = {e: k for k, e in enumerate(edges)}
        ref_faces = [(slot[seq[3 * k + 2]], slot[seq[3 * k + 1]], slot[seq[3 * k]])
                     for k in range(len(seq) // 3)]
        assert ref_faces == faces, ('faces', c)


def mt_cases(t):
    """Per case (MT corner order): emitted faces as voxel-edge ids (0..18).

    Mirrors tetIx (src/marching_tetrahedra.jl:11-18), voxEdgeId (:91-95) and
    procVox (:105-127): tets 1..6, skip tet cases 0 and 15, one or two faces
    from tetTri, vertex ids evaluated left to right.
    """
    sub, mask = t['subTets'], t['subTetsMask']
    tec, ttri, vix = t['tetEdgeCrnrs'], t['tetTri'], t['voxEdgeIx']

    def vox_edge(i, te):
        a = sub[i][tec[te - 1][0] - 1]
        b = sub[i][tec[te - 1][1] - 1]
        e = vix[a - 1][b - 1]
        assert e != 0
        return e - 1

    cases = []
    for c in range(256):
        faces = []
        if c not in (0, 255):
            for i in range(6):
                ix = (c & 0x01) | ((c & 0x40) >> 3)
                if mask[i][0] & c:
                    ix |= 0x02
                if mask[i][1] & c:
                    ix |= 0x04
                if ix in (0, 15):
                    continue
                e = ttri[ix - 1]
                faces.append((vox_edge(i, e[0]), vox_edge(i, e[1]), vox_edge(i, e[2])))
                if e[3] != 0:
                    faces.append((vox_edge(i, e[3]), vox_edge(i, e[4]), vox_edge(i, e[5])))
        cases.append(faces)
    return cases


def check_mt(t, cases):
    pos = t['voxCrnrPos']
    ecr = t['voxEdgeCrnrs']
    for c in range(256):
        crossed = set()
        for e in range(19):
            a, b = ecr[e][0] - 1, ecr[e][1] - 1
            if ((c >> a) & 1) != ((c >> b) & 1):
                crossed.add(e)
        used = {e for f in cases[c] for e in f}
        assert used == crossed, ('MT emitted edges must be exactly the crossed ones', c)
        # every edge runs from its lower corner to its upper corner
    for e in range(19):
        a, b = pos[ecr[e][0] - 1], pos[ecr[e][1] - 1]
        assert all(bb >= aa for aa, bb in zip(a, b)) and a != b
    # subTetsMask holds the bits of tet corners 2 and 3
    for i in range(6):
        assert t['subTetsMask'][i][0] == 1 << (t['subTets'][i][1] - 1)
        assert t['subTetsMask'][i][1] == 1 << (t['subTets'][i][2] - 1)


def emit(out, mc, mt_t, mt):
    L = []
    w = L.append
    w('// Generated by gen_tables.py from Meshing.jl v0.7.0 src/lut/mc.jl and src/lut/mt.jl.')
    w('// Do not edit by hand.  Every cube case 0..255 is flattened into the exact')
    w('// vertex / face emission sequence of process_mc_voxel! (src/marching_cubes.jl:67-92)')
    w('// and procVox (src/marching_tetrahedra.jl:105-127).')
    w('#pragma once')
    w('#include <stdint.h>')
    w('// Storage class of the tables; device code defines it as `static __device__ const`.')
    w('#ifndef MESH_TBL')
    w('#define MESH_TBL static const')
    w('#endif')
    w('')
    w('// ---- Marching Cubes (corner order of src/marching_cubes.jl:42-49) ----')
    w('// MC_CASE_VERTS[c]: nibble k (bits 4k..4k+3) = cube edge (0..11) of local vertex slot k;')
    w('// bits 48..51 = number of vertices, bits 52..54 = number of faces.')
    w('// MC_CASE_FACES[c]: face f in bits 12f..12f+11 = three 4-bit local slots (s0 | s1<<4 | s2<<8),')
    w('// in emission order; the emitted face is (base+s0+1, base+s1+1, base+s2+1).')
    vw, fw = [], []
    maxnv = maxnf = 0
    for c in range(256):
        edges, faces = mc[c]
        v = 0
        for k, e in enumerate(edges):
            v |= e << (4 * k)
        v |= len(edges) << 48
        v |= len(faces) << 52
        f = 0
        for k, (a, b, cc) in enumerate(faces):
            f |= (a | (b << 4) | (cc << 8)) << (12 * k)
        vw.append(v)
        fw.append(f)
        maxnv = max(maxnv, len(edges))
        maxnf = max(maxnf, len(faces))
    w('#define MC_MAX_VERTS %d' % maxnv)
    w('#define MC_MAX_FACES %d' % maxnf)
    w('MESH_TBL uint64_t MC_CASE_VERTS[256] = {')
    for i in range(0, 256, 4):
        w('  ' + ', '.join('0x%016xull' % x for x in vw[i:i + 4]) + ',')
    w('};')
    w('MESH_TBL uint64_t MC_CASE_FACES[256] = {')
    for i in range(0, 256, 4):
        w('  ' + ', '.join('0x%016xull' % x for x in fw[i:i + 4]) + ',')
    w('};')
    w('')
    w('// ---- Marching Tetrahedra (corner order of src/marching_tetrahedra.jl:146-153) ----')
    w('// MT_CASE_FACES[c][3f+k]: voxel edge (0..18) of vertex k of face f, emission order.')
    w('// MT_CASE_NFACES[c]: number of faces.  MT_TOUCHED[c]: 19-bit mask of edges used.')
    w('// MT_TOUCH_ORDER[c][r]: r-th distinct edge in first-use order (0xff past the end).')
    maxf = max(len(f) for f in mt)
    orders = []
    for c in range(256):
        seen = []
        for f in mt[c]:
            for e in f:
                if e not in seen:
                    seen.append(e)
        orders.append(seen)
    maxt = max(len(o) for o in orders)
    w('#define MT_MAX_FACES %d' % maxf)
    w('#define MT_MAX_TOUCH %d' % maxt)
    w('MESH_TBL uint8_t MT_CASE_NFACES[256] = {')
    for i in range(0, 256, 16):
        w('  ' + ', '.join('%d' % len(mt[c]) for c in range(i, i + 16)) + ',')
    w('};')
    w('MESH_TBL uint8_t MT_CASE_FACES[256][%d] = {' % (3 * maxf))
    for c in range(256):
        flat = [e for f in mt[c] for e in f]
        flat += [0xff] * (3 * maxf - len(flat))
        w('  {' + ','.join('%d' % e for e in flat) + '},')
    w('};')
    w('MESH_TBL uint32_t MT_TOUCHED[256] = {')
    for i in range(0, 256, 8):
        w('  ' + ', '.join('0x%05xu' % sum(1 << e for e in orders[c]) for c in range(i, i + 8)) + ',')
    w('};')
    w('MESH_TBL uint8_t MT_TOUCH_ORDER[256][%d] = {' % maxt)
    for c in range(256):
        o = orders[c] + [0xff] * (maxt - len(orders[c]))
        w('  {' + ','.join('%d' % e for e in o) + '},')
    w('};')
    w('// MT_BEFORE[c][e]: mask of the edges first used before edge e in case c (0 if e is unused).')
    w('MESH_TBL uint32_t MT_BEFORE[256][19] = {')
    for c in range(256):
        o = orders[c]
        row = []
        for e in range(19):
            row.append(sum(1 << x for x in o[:o.index(e)]) if e in o else 0)
        w('  {' + ','.join('0x%05xu' % m for m in row) + '},')
    w('};')
    w('')
    w('// Voxel geometry restated from src/lut/mt.jl:23-56 (0-based corners).')
    w('MESH_TBL uint8_t MT_CORNER_POS[8][3] = {' +
      ', '.join('{%d,%d,%d}' % tuple(p) for p in mt_t['voxCrnrPos']) + '};')
    w('MESH_TBL uint8_t MT_EDGE_CORNERS[19][2] = {' +
      ', '.join('{%d,%d}' % (a - 1, b - 1) for a, b in mt_t['voxEdgeCrnrs']) + '};')
    w('MESH_TBL uint8_t MT_EDGE_DIR[19] = {' + ', '.join('%d' % d for d in mt_t['voxEdgeDir']) + '};')
    w('')
    open(out, 'w').write('\n'.join(L) + '\n')


def main():
    if len(sys.argv) != 2:
        sys.exit('usage: %s <Meshing.jl checkout>' % sys.argv[0])
    ref = sys.argv[1]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'mesh_tables.h')
    verts, eqmap, conn, elist, tri = load_mc(ref)
    # edge list restated in the kernels must match the reference's (_mc_edge_list)
    assert [tuple(e) for e in elist] == [(1, 2), (2, 3), (3, 4), (4, 1), (5, 6), (6, 7), (7, 8),
                                         (8, 5), (1, 5), (2, 6), (3, 7), (4, 8)]
    mc = mc_cases(verts, eqmap, conn)
    check_mc_against_tri_table(mc, tri)
    mt_t = load_mt(ref)
    mt = mt_cases(mt_t)
    check_mt(mt_t, mt)
    emit(out, mc, mt_t, mt)
    print('wrote', out)


if __name__ == '__main__':
    main()
