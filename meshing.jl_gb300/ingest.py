"""Volume ingest: NRRD and raw files into host or device volumes.

The reference's CT example (examples/nrrd.jl) loads an NRRD file through
FileIO/NRRD.jl and passes the array to ``isosurface`` with the default
X = Y = Z = -1:1.  ``read_nrrd`` returns the same array (Julia layout: the
first NRRD axis is x, fastest in memory) plus the physical axis ranges the
header describes, for callers that want them:

    A, hdr = read_nrrd('CTA-cardio.nrrd')                  # numpy, indexed A[x, y, z]
    verts, faces = isosurface(A, MarchingTetrahedra(iso=100))
    V, hdr = read_nrrd('CTA-cardio.nrrd', device='cuda')   # CUDA tensor through pinned staging

Supported: NRRD0001-0005 headers; types (u)int8, int16, uint16, int32, int64,
float (Float32), double (Float64); encodings raw, gzip, bzip2, ascii; little
and big endian; attached data or one detached data file; ``byte skip`` and
``line skip``.  Volumes must be 3-D (a 4-D header with a leading size-1 axis
is accepted).  Element types the engine cannot take (uint32, uint64, block)
raise ValueError, as do multi-file data lists.
"""
import bz2
import gzip
import os
import zlib

import numpy as np

_TYPES = {
    'signed char': np.int8, 'int8': np.int8, 'int8_t': np.int8,
    'uchar': np.uint8, 'unsigned char': np.uint8, 'uint8': np.uint8, 'uint8_t': np.uint8,
    'short': np.int16, 'short int': np.int16, 'signed short': np.int16, 'signed short int': np.int16,
    'int16': np.int16, 'int16_t': np.int16,
    'ushort': np.uint16, 'unsigned short': np.uint16, 'unsigned short int': np.uint16, 'uint16': np.uint16,
    'uint16_t': np.uint16,
    'int': np.int32, 'signed int': np.int32, 'int32': np.int32, 'int32_t': np.int32,
    'longlong': np.int64, 'long long': np.int64, 'long long int': np.int64, 'signed long long': np.int64,
    'signed long long int': np.int64, 'int64': np.int64, 'int64_t': np.int64,
    'float': np.float32, 'double': np.float64,
}
_UNSUPPORTED = {'uint', 'unsigned int', 'uint32', 'uint32_t', 'ulonglong', 'unsigned long long',
                'unsigned long long int', 'uint64', 'uint64_t', 'block'}


class NrrdHeader(dict):
    """The header's fields (lower-case keys) plus the derived ``shape`` (nx, ny,
    nz), ``dtype`` and ``ranges``: ((x0, x1), (y0, y1), (z0, z1)) in world units
    when the header gives axis-aligned spacing (``space directions``,
    ``spacings`` or ``axis mins`` / ``axis maxs``), else None."""


def _parse_vector(s):
    s = s.strip()
    if s == 'none':
        return None
    return [float(t) for t in s.strip('()').split(',')]


def _parse_header(f):
    magic = f.readline()
    if not magic.startswith(b'NRRD000'):
        raise ValueError('not an NRRD file')
    hdr = NrrdHeader()
    while True:
        line = f.readline()
        if not line:
            break  # detached header: no data follows
        line = line.rstrip(b'\r\n').decode('latin-1')
        if line == '':
            break
        if line.startswith('#'):
            continue
        if ':=' in line:  # key/value pair: kept as is
            k, v = line.split(':=', 1)
            hdr.setdefault('keyvalue', {})[k] = v
            continue
        if ': ' not in line:
            raise ValueError('malformed NRRD header line %r' % line)
        k, v = line.split(': ', 1)
        hdr[k.strip().lower()] = v.strip()
    return hdr


def _axis_ranges(hdr, sizes):
    spacing = origin = None
    if 'space directions' in hdr:
        vecs = [_parse_vector(t) for t in hdr['space directions'].replace(') (', ')|(').split('|')]
        vecs = [v for v in vecs if v is not None]
        if len(vecs) == 3 and all(sum(1 for c in v if c != 0) == 1 for v in vecs) and \
                all(v[i] != 0 for i, v in enumerate(vecs)):
            spacing = [v[i] for i, v in enumerate(vecs)]
        if 'space origin' in hdr:
            origin = _parse_vector(hdr['space origin'])
    elif 'spacings' in hdr:
        sp = [float(t) for t in hdr['spacings'].split() if t.lower() != 'nan']
        if len(sp) == 3:
            spacing = sp
    if spacing is None and 'axis mins' in hdr and 'axis maxs' in hdr:
        lo = [float(t) for t in hdr['axis mins'].split()][-3:]
        hi = [float(t) for t in hdr['axis maxs'].split()][-3:]
        return tuple((a, b) for a, b in zip(lo, hi))
    if spacing is None:
        return None
    origin = origin or [0.0, 0.0, 0.0]
    return tuple((o, o + (s - 1) * d) for o, s, d in zip(origin, sizes[-3:], spacing))


def read_nrrd_header(path):
    """The parsed header of an NRRD file (see NrrdHeader)."""
    with open(path, 'rb') as f:
        hdr = _parse_header(f)
        hdr['_data_offset'] = f.tell()
    tname = hdr.get('type', '').lower()
    if tname in _UNSUPPORTED:
        raise ValueError('NRRD type %r has no engine kernel' % tname)
    if tname not in _TYPES:
        raise ValueError('unknown NRRD type %r' % tname)
    sizes = [int(t) for t in hdr['sizes'].split()]
    if int(hdr.get('dimension', len(sizes))) != len(sizes):
        raise ValueError('dimension and sizes disagree')
    if len(sizes) == 4 and sizes[0] == 1:
        sizes = sizes[1:]
    if len(sizes) != 3:
        raise ValueError('only 3-D volumes are meshed (sizes %s)' % hdr['sizes'])
    dt = np.dtype(_TYPES[tname])
    endian = hdr.get('endian', 'little').lower()
    if dt.itemsize > 1:
        dt = dt.newbyteorder('<' if endian == 'little' else '>')
    hdr['shape'] = tuple(sizes)
    hdr['dtype'] = dt
    hdr['ranges'] = _axis_ranges(hdr, sizes)
    return hdr


def _payload(path, hdr):
    """The (decoded) data bytes of the volume."""
    datafile = hdr.get('data file', hdr.get('datafile'))
    if datafile is not None:
        if datafile.startswith('LIST') or len(datafile.split()) > 1:
            raise ValueError('multi-file NRRD data is not supported')
        src = os.path.join(os.path.dirname(os.path.abspath(path)), datafile)
        offset = 0
    else:
        src, offset = path, hdr['_data_offset']
    with open(src, 'rb') as f:
        f.seek(offset)
        for _ in range(int(hdr.get('line skip', hdr.get('lineskip', 0)))):
            f.readline()
        raw = f.read()
    enc = hdr.get('encoding', 'raw').lower()
    nbytes = int(np.prod(hdr['shape'])) * hdr['dtype'].itemsize
    skip = int(hdr.get('byte skip', hdr.get('byteskip', 0)))
    if enc in ('gzip', 'gz'):
        raw = zlib.decompressobj(zlib.MAX_WBITS | 16).decompress(raw)
    elif enc in ('bzip2', 'bz2'):
        raw = bz2.decompress(raw)
    elif enc in ('ascii', 'text', 'txt'):
        vals = np.array(raw.split())  # text tokens, converted exactly (no float detour for integers)
        if vals.size != np.prod(hdr['shape']):
            raise ValueError('ascii data holds %d values, not %d' % (vals.size, np.prod(hdr['shape'])))
        return vals.astype(hdr['dtype']).tobytes()
    elif enc != 'raw':
        raise ValueError('NRRD encoding %r is not supported' % enc)
    if skip == -1:
        raw = raw[len(raw) - nbytes:]
    else:
        raw = raw[skip:]
    if len(raw) < nbytes:
        raise ValueError('NRRD data holds %d bytes, the header needs %d' % (len(raw), nbytes))
    return raw[:nbytes]


def read_nrrd(path, device=None):
    """(A, header): A indexed A[x, y, z] (first NRRD axis = x, fastest in memory),
    native byte order; a numpy array, or a CUDA tensor (Julia layout) when
    ``device`` is given, staged through pinned host memory."""
    hdr = read_nrrd_header(path)
    data = _payload(path, hdr)
    nx, ny, nz = hdr['shape']
    arr = np.frombuffer(data, dtype=hdr['dtype']).reshape((nz, ny, nx))
    if not hdr['dtype'].isnative:
        arr = arr.astype(hdr['dtype'].newbyteorder('='))
    if device is None:
        return np.asfortranarray(arr.transpose(2, 1, 0)), hdr
    return to_device(arr, device), hdr


def to_device(zyx, device='cuda'):
    """A [z][y][x] C-order numpy array as a CUDA tensor indexed [x, y, z] (Julia
    layout), copied from pinned host memory."""
    import torch
    tdt = torch.from_numpy(np.empty(0, dtype=zyx.dtype)).dtype
    host = torch.empty(zyx.shape, dtype=tdt, pin_memory=True)
    host.numpy()[...] = zyx  # one copy, straight into pinned memory
    dev = host.to(device, non_blocking=True)
    torch.cuda.current_stream(dev.device).synchronize()
    return dev.permute(2, 1, 0)


def read_raw(path, shape, dtype, offset=0, endian='little', device=None):
    """A headerless volume of ``shape`` (nx, ny, nz), x fastest in the file."""
    dt = np.dtype(dtype)
    if dt.itemsize > 1:
        dt = dt.newbyteorder('<' if endian == 'little' else '>')
    nx, ny, nz = shape
    arr = np.fromfile(path, dtype=dt, count=nx * ny * nz, offset=offset)
    if arr.size != nx * ny * nz:
        raise ValueError('raw file holds %d values, not %d' % (arr.size, nx * ny * nz))
    arr = arr.reshape((nz, ny, nx))
    if not dt.isnative:
        arr = arr.astype(dt.newbyteorder('='))
    if device is None:
        return np.asfortranarray(arr.transpose(2, 1, 0))
    return to_device(arr, device)


def write_nrrd(path, A, encoding='raw', detached=False, endian='little', spacing=None, origin=None):
    """Writes A (indexed A[x, y, z]) as an NRRD0004 file; the inverse of read_nrrd."""
    A = np.asarray(A)
    tname = {'int8': 'int8', 'uint8': 'uint8', 'int16': 'int16', 'uint16': 'uint16', 'int32': 'int32',
             'int64': 'int64', 'float32': 'float', 'float64': 'double'}[A.dtype.name]
    dt = A.dtype.newbyteorder('<' if endian == 'little' else '>') if A.dtype.itemsize > 1 else A.dtype
    zyx = np.ascontiguousarray(A.transpose(2, 1, 0)).astype(dt)
    if encoding == 'ascii':
        body = ' '.join(repr(v.item()) for v in zyx.ravel()).encode() + b'\n'
    else:
        body = zyx.tobytes()
        if encoding == 'gzip':
            body = gzip.compress(body)
        elif encoding == 'bzip2':
            body = bz2.compress(body)
    lines = ['NRRD0004', 'type: %s' % tname, 'dimension: 3', 'sizes: %d %d %d' % A.shape,
             'encoding: %s' % encoding]
    if A.dtype.itemsize > 1:
        lines.append('endian: %s' % endian)
    if spacing is not None:
        lines.append('space: right-anterior-superior')
        lines.append('space directions: (%r,0,0) (0,%r,0) (0,0,%r)' % tuple(float(s) for s in spacing))
        if origin is not None:
            lines.append('space origin: (%r,%r,%r)' % tuple(float(o) for o in origin))
    if detached:
        data_name = os.path.basename(path) + ('.raw' if encoding == 'raw' else '.' + encoding)
        lines.append('data file: %s' % data_name)
        with open(os.path.join(os.path.dirname(os.path.abspath(path)), data_name), 'wb') as f:
            f.write(body)
        with open(path, 'w') as f:
            f.write('\n'.join(lines) + '\n')
    else:
        with open(path, 'wb') as f:
            f.write(('\n'.join(lines) + '\n\n').encode())
            f.write(body)
    return path


__all__ = ['read_nrrd', 'read_nrrd_header', 'read_raw', 'write_nrrd', 'to_device', 'NrrdHeader']
