#!/usr/bin/env python3
"""Write ``ref_luts.h`` for the CPU oracle (test infrastructure only).

The oracle walks the lookup tables in the reference's own structure, the way
``process_mc_voxel!`` (src/marching_cubes.jl:67-92) and ``procVox``
(src/marching_tetrahedra.jl:105-127) do, so that the product's flattened
per-case tables (meshing.jl_gb300/csrc/mesh_tables.h) are checked against an
independent walk.  Tables: ``_mc_verts``, ``_mc_eq_mapping``,
``_mc_connectivity``, ``_mc_edge_list`` (src/lut/mc.jl:301-608) and the MT
tables of src/lut/mt.jl:23-107, kept 1-based with 0 as terminator like the
reference.  Run by hand with the reference checkout as argv[1]; the output is
committed.
"""
import os
import re
import sys


def grab(src, name):
    i = src.index('const ' + name)
    j = src.find('\nconst', i + 1)
    body = src[i:j if j > 0 else len(src)]
    return '\n'.join(line.split('#')[0] for line in body.split('\n'))


def rows(body):
    inner = body[body.index('(') + 1:]
    return [[int(x, 0) for x in r.replace(' ', '').replace('\n', '').split(',') if x]
            for r in re.findall(r'\(([^()]*)\)', inner)]


def flat(body):
    return [int(x, 16) for x in re.findall(r'0x[0-9a-f]+', body)]


def c_array(name, ctype, data):
    if isinstance(data[0], list):
        inner = ',\n  '.join('{' + ','.join(str(v) for v in r) + '}' for r in data)
        return 'static const %s %s[%d][%d] = {\n  %s\n};' % (ctype, name, len(data), len(data[0]), inner)
    return 'static const %s %s[%d] = {%s};' % (ctype, name, len(data), ','.join(str(v) for v in data))


def main():
    if len(sys.argv) != 2:
        sys.exit('usage: %s <Meshing.jl checkout>' % sys.argv[0])
    ref = sys.argv[1]
    mc = open(os.path.join(ref, 'src/lut/mc.jl')).read()
    mt = open(os.path.join(ref, 'src/lut/mt.jl')).read()
    out = ['// Generated by gen_ref_luts.py from Meshing.jl v0.7.0 src/lut/mc.jl and src/lut/mt.jl.',
           '// Oracle (test infrastructure) copy of the lookup tables in the reference layout:',
           '// 1-based entries, 0 terminates a row.  Do not edit by hand.',
           '#pragma once', '#include <stdint.h>']
    out.append(c_array('R_MC_VERTS', 'uint8_t', rows(grab(mc, '_mc_verts'))))
    out.append(c_array('R_MC_EQ_MAPPING', 'uint8_t', flat(grab(mc, '_mc_eq_mapping'))))
    out.append(c_array('R_MC_CONNECTIVITY', 'uint8_t', rows(grab(mc, '_mc_connectivity'))))
    out.append(c_array('R_MC_EDGE_LIST', 'uint8_t', rows(grab(mc, '_mc_edge_list'))))
    for name, ctype in (('voxCrnrPos', 'int64_t'), ('voxEdgeCrnrs', 'uint8_t'), ('voxEdgeIx', 'uint8_t'),
                        ('subTets', 'uint8_t'), ('subTetsMask', 'uint8_t'), ('tetEdgeCrnrs', 'uint8_t'),
                        ('tetTri', 'uint8_t')):
        out.append(c_array('R_' + name, ctype, rows(grab(mt, name))))
    out.append(c_array('R_voxEdgeDir', 'int64_t', flat(grab(mt, 'voxEdgeDir'))))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'ref_luts.h')
    open(path, 'w').write('\n'.join(out) + '\n')
    print('wrote', path)


if __name__ == '__main__':
    main()
