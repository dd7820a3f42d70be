"""GB300 isosurface engine with Meshing.jl's API.

Python mirror of the reference interface (src/Meshing.jl:9-11 exports
``isosurface``, ``MarchingCubes``, ``MarchingTetrahedra``; NaiveSurfaceNets is
named in README.md:21 and defined here):

    points, faces = isosurface(A)                                  # MarchingCubes()
    points, faces = isosurface(A, MarchingCubes(iso=0.5))
    points, faces = isosurface(A, MarchingTetrahedra(iso=0.5, eps=1e-3), X, Y, Z)

``A`` is indexed A[x, y, z] like a Julia array (x fastest in memory); the
Julia type of ``iso``/``eps``/range endpoints follows the Python type
(int -> Int64, float -> Float64, numpy.float32 -> Float32).  Every call runs
on the GPU through the C ABI (include/meshing_gb300.h); there is no CPU path.
"""
from ._lib import Context, MeshError, MeshParams, load as load_library
from .api import (MarchingCubes, MarchingTetrahedra, NaiveSurfaceNets, AbstractMeshingAlgorithm, isosurface,
                  isosurface_device, isosurface_slabs, output_float_bits, make_params, default_context)
from .batch import Batch
from .serve import Server
from . import export, ingest

__all__ = ['isosurface', 'isosurface_device', 'isosurface_slabs', 'MarchingCubes', 'MarchingTetrahedra', 'NaiveSurfaceNets',
           'AbstractMeshingAlgorithm', 'MeshError', 'Context', 'MeshParams', 'output_float_bits', 'make_params',
           'default_context', 'load_library', 'Batch', 'Server', 'export', 'ingest']
