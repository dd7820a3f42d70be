"""Build the CUDA engine into ``_build/libmeshing_gb300.so`` (sm_103a only).

Translation units are compiled in parallel with nvcc and linked into one
shared library exporting the C ABI of include/meshing_gb300.h.  Device code
is built with ``-fmad=false`` and host code with ``-ffp-contract=off`` so that
no multiply-add is fused: the reference's arithmetic rounds every operation.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'libmeshing_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
SOURCES = ['mesh_api.cu', 'k_tables.cu', 'k_classify.cu', 'k_scan.cu', 'k_walk_mc.cu', 'k_emit_mc.cu',
           'k_direct_mc.cu', 'k_emit_halo.cu', 'mesh_noalloc.cu', 'mesh_batch.cu', 'mesh_serve.cu', 'k_post.cu', 'k_weld.cu']


def nvcc():
    exe = shutil.which('nvcc')
    if exe:
        return exe
    cand = '/usr/local/cuda/bin/nvcc'
    if os.path.exists(cand):
        return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build meshing_gb300')


def _flags():
    return ARCH + ['-O3', '-lineinfo', '-std=c++17', '-fmad=false', '-Xcompiler', '-fPIC', '-Xcompiler',
                   '-ffp-contract=off', '-Xcompiler', '-fvisibility=hidden', '-I', CSRC,
                   '-I', os.path.join(HERE, '..', 'include')]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cu', '.cuh', '.h'))]
    files.append(os.path.join(HERE, '..', 'include', 'meshing_gb300.h'))
    files.append(os.path.abspath(__file__))
    return files


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force=False, verbose=False, extra=()):
    """Compile if sources changed; returns the library path."""
    if not force and not stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    tag = str(os.getpid())

    def one(src):
        obj = os.path.join(BUILD, src.replace('.cu', '.%s.o' % tag))
        cmd = [cc] + _flags() + list(extra) + ['-c', os.path.join(CSRC, src), '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, ' '.join(cmd), r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + '.' + tag
    cmd = [cc] + ARCH + ['-shared', '-o', tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    for o in objs:
        os.remove(o)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s' % r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    import sys
    print(build(force='--force' in sys.argv, verbose=True,
                extra=['-Xptxas', '-v'] if '--ptxas' in sys.argv else []))
