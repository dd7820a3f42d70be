/*
 * meshing_gb300.h -- C ABI of the GB300 isosurface engine.
 *
 * Drop-in device back end for Meshing.jl's `isosurface(A, alg, X, Y, Z)`:
 *   - MarchingCubes       replaces src/marching_cubes.jl:27-64 (with :67-120)
 *   - MarchingTetrahedra  replaces src/marching_tetrahedra.jl:129-163 (with :11-127)
 *   - NaiveSurfaceNets    named by the reference (README.md:21) but not
 *                         implemented there; defined by this project.
 * The algorithm structs (src/algorithmtypes.jl:23-25,37-40) map onto
 * `mesh_params`; the generic forwarder `isosurface(A, args...)`
 * (src/isosurface.jl:30-32) stays on the Julia side.
 *
 * Results are those of the reference: vertices `NTuple{3, float(FT)}` with
 * FT = promote_type(eltype(first(X)), eltype(first(Y)), eltype(first(Z)),
 * eltype(A), typeof(iso)[, typeof(eps)]), faces `NTuple{3, Int}` with 1-based
 * indices, both in the reference's emission order.
 *
 * The volume uses Julia's column-major layout: A[x, y, z] is element
 * x + nx*(y + ny*z) (0-based).  No function throws; every function returns a
 * `mesh_status`.  A context is not thread-safe; use one context per thread.
 */
#ifndef MESHING_GB300_H
#define MESHING_GB300_H

#include <stdint.h>

#ifndef MESH_API
#define MESH_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Element types (volume, iso, eps, range endpoints). */
typedef enum {
    MESH_DT_U16 = 1, /* UInt16 */
    MESH_DT_F32 = 2, /* Float32 */
    MESH_DT_F64 = 3, /* Float64 */
    MESH_DT_I64 = 4, /* Int64 */
    MESH_DT_I32 = 5, /* Int32 (volumes only) */
    MESH_DT_F16 = 6, /* Float16 (volumes only; iso of type Float32 or Float64) */
    MESH_DT_I16 = 7, /* Int16 (volumes only) */
    MESH_DT_I8 = 8,  /* Int8 (volumes only) */
    MESH_DT_U8 = 9   /* UInt8 (volumes only) */
} mesh_dtype;

typedef enum {
    MESH_ALG_MC = 0,  /* MarchingCubes       (src/algorithmtypes.jl:23-25) */
    MESH_ALG_MT = 1,  /* MarchingTetrahedra  (src/algorithmtypes.jl:37-40) */
    MESH_ALG_NSN = 2, /* NaiveSurfaceNets    (defined by this project) */
    /* MarchingCubes with one vertex per crossed lattice edge (opt-in, not a
     * drop-in: the reference pushes a vertex per cell and edge,
     * src/marching_cubes.jl:72-79).  Vertices are numbered when their edge is
     * first met -- cells in the reference's emission order, a cell's edges in
     * its vertex-slot order -- and placed by that cell's vertex_interp; faces
     * are the reference's triangles on those ids.  mesh_count / mesh_fill only. */
    MESH_ALG_MC_WELDED = 3
} mesh_alg;

typedef enum {
    MESH_OK = 0,
    MESH_EINVAL = 1,       /* bad argument (null pointer, unsupported type, non-finite range, ...) */
    MESH_ENOMEM = 2,       /* device or pinned-host allocation failed */
    MESH_ECUDA = 3,        /* a CUDA runtime call failed */
    MESH_EDEVICE = 4,      /* a kernel reported an error (bounded wait expired, bounds check) */
    MESH_ESTATE = 5,       /* mesh_fill without a preceding successful mesh_count */
    MESH_ECAPACITY = 6,    /* output buffers smaller than the mesh */
    MESH_ETOOLARGE = 7,    /* volume beyond the engine's index limits (more than 2^21 samples on x or z,
                              more than 2^21 - 31 on y) */
    MESH_ESCRATCH = 8,     /* mesh_extract_noalloc: the call needs more than MESH_NOALLOC_SCRATCH_BYTES */
    MESH_EBUDGET = 9,      /* mesh_server_submit: the request's worst case exceeds the memory budget */
    MESH_EBUSY = 10        /* mesh_server_submit: the queue is full */
} mesh_status;

/* Mirrors MarchingCubes{T}(iso) / MarchingTetrahedra{T,E}(iso, eps) plus the
 * X, Y, Z arguments of isosurface.  Each scalar travels as a double together
 * with its Julia type; Int64 values must satisfy |v| <= 2^53. */
typedef struct {
    int32_t alg;        /* mesh_alg */
    int32_t iso_type;   /* MESH_DT_F32 | MESH_DT_F64 | MESH_DT_I64 (not I64 with MESH_DT_F16 volumes) */
    double iso;
    int32_t eps_type;   /* MESH_DT_F32 | MESH_DT_F64 (MT only; ignored otherwise) */
    double eps;
    int32_t range_type; /* eltype of first(X) == first(Y) == first(Z): MESH_DT_I64 | F32 | F64 */
    double range[6];    /* first(X), last(X), first(Y), last(Y), first(Z), last(Z) */
} mesh_params;

/* Fills `p` with the reference defaults: MarchingCubes(iso=0.0), eps=1e-3,
 * X = Y = Z = -1:1 (src/algorithmtypes.jl:23-25,37-40; src/marching_cubes.jl:27). */
MESH_API void mesh_params_default(mesh_params *p);

typedef struct mesh_ctx mesh_ctx;

/* Creates a context bound to CUDA device `device` with its own stream. */
MESH_API int mesh_ctx_create(int device, mesh_ctx **out);
MESH_API void mesh_ctx_destroy(mesh_ctx *ctx);
/* Makes the context issue its work on `stream` (a cudaStream_t; NULL = the context's own).
   Host-buffer calls on volumes or meshes of at least MESHING_GB300_PIPELINE_BYTES (default
   256 MiB; 0 = never) also use a second, internal copy stream, ordered against `stream` by
   events: mesh_count uploads in groups of z segments, each classified on arrival, and
   mesh_fill downloads a Marching Cubes mesh in x ranges while the next range is emitted.
   Both calls still return only when their work is complete. */
MESH_API int mesh_ctx_set_stream(mesh_ctx *ctx, void *stream);
/* No counterpart in the reference.  Until reset with (0, 0, 0), the volumes of
 * the context's calls are x samples x_first .. x_first+nx-1 of a volume whose x
 * axis has nx_total samples: node coordinates are those of LinRange(first(X),
 * last(X), nx_total), so an x slab meshes exactly as that part of the whole
 * volume (x is the outermost emission axis: slab meshes concatenate into the
 * whole one, face indices offset by the vertices before them).  Marching Cubes
 * slabs of cells [c0, c1) pass samples c0 .. c1 with halo = 0.  Marching
 * Tetrahedra and Naive Surface Nets share vertices across the boundary, which
 * belong to the lower cell column: every slab after the first passes samples
 * c0-1 .. c1 with x_first = c0-1 and halo = 1; its first cell column (the
 * previous slab's last) is counted but not emitted, mesh_count returns the
 * counts without it, and faces that use the previous slab's vertices have
 * indices <= 0 before the offset is added.  With halo = 1, mesh_extract_device
 * returns MESH_EINVAL, and so does a Marching Cubes call. */
MESH_API int mesh_set_x_window(mesh_ctx *ctx, int64_t x_first, int64_t nx_total, int halo);
MESH_API const char *mesh_status_string(int status);
/* Last error message recorded on `ctx` (empty string if none). */
MESH_API const char *mesh_ctx_last_error(const mesh_ctx *ctx);

/* Bits (32 or 64) of float(FT) for a volume of `vol_dtype` under `p`. */
MESH_API int mesh_output_float_bits(int vol_dtype, const mesh_params *p, int *bits);

/* Phase 1 of the two-phase drop-in call (replaces the loops of
 * src/marching_cubes.jl:40-63 / src/marching_tetrahedra.jl:144-160):
 * classifies every cell and scans the per-column counts.  `vol` is a host
 * pointer (vol_on_device = 0, copied in by the library) or a device pointer
 * (vol_on_device = 1, must stay valid until mesh_fill returns).  Blocks until
 * the counts are known. */
MESH_API int mesh_count(mesh_ctx *ctx, const void *vol, int vol_dtype, int64_t nx, int64_t ny, int64_t nz,
               int vol_on_device, const mesh_params *p, int64_t *nverts, int64_t *nfaces);

/* Phase 2: writes exactly nverts*3 floats (float or double, per
 * mesh_output_float_bits) to `verts` and nfaces*3 int64 (1-based) to `faces`,
 * host pointers (out_on_device = 0) or device pointers (1).  Blocks until done. */
MESH_API int mesh_fill(mesh_ctx *ctx, void *verts, int64_t *faces, int out_on_device);

/* Device-resident single call, asynchronous on the context stream: classify,
 * scan and emit with no host round trip.  `vol`, `verts`, `faces` and
 * `counts` are device pointers; counts[0] = nverts and counts[1] = nfaces are
 * written on the device.  If the mesh exceeds verts_cap / faces_cap nothing
 * beyond the capacities is written and mesh_ctx_sync() returns MESH_ECAPACITY;
 * counts still hold the true sizes. */
MESH_API int mesh_extract_device(mesh_ctx *ctx, const void *vol, int vol_dtype, int64_t nx, int64_t ny, int64_t nz,
                        const mesh_params *p, void *verts, int64_t verts_cap, int64_t *faces, int64_t faces_cap,
                        int64_t *counts);
/* Waits for the context's outstanding work and reports device-side errors. */
MESH_API int mesh_ctx_sync(mesh_ctx *ctx);

/* No counterpart in Meshing.jl (post-processing of a finished mesh, the
 * published area-weighted rule of GeometryBasics' normals(vertices, faces)):
 * normal i = normalize(sum over the faces f using vertex i of
 * cross(v[f2] - v[f1], v[f3] - v[f1])), accumulated in Float64 and written in
 * the vertex type; a vertex on no face of non-zero area gets (0, 0, 0).
 * `verts` (nverts x 3, float_bits 32 or 64), `faces` (nfaces x 3, 1-based) and
 * `normals` (nverts x 3, the vertex type) are device pointers.  Asynchronous on
 * the context stream; mesh_ctx_sync() reports MESH_EDEVICE if a face index
 * lies outside 1..nverts (that face is skipped).  Uses the context's error word:
 * a two-phase call in progress must finish (mesh_fill) first. */
MESH_API int mesh_vertex_normals(mesh_ctx *ctx, const void *verts, int float_bits, int64_t nverts,
                                 const int64_t *faces, int64_t nfaces, void *normals);

/* Diagnostics (no counterpart in the reference, which has no instrumentation):
 * with timing enabled the context brackets every kernel launch with CUDA
 * events on its stream.  mesh_ctx_stage_times waits for them and returns, per
 * stage -- 0 classify, 1 scan, 2 emit (the Marching Cubes active-cell
 * compaction, or the whole MT / NSN emit), 3 Marching Cubes expansion -- the
 * summed device milliseconds ms[0..3] and the number of kernel launches
 * launches[0..3] since the previous query (the coordinate-table kernel counts
 * with stage 0, the four scan kernels with stage 1), then resets. */
MESH_API int mesh_ctx_enable_timing(mesh_ctx *ctx, int enable);
MESH_API int mesh_ctx_stage_times(mesh_ctx *ctx, double *ms, int64_t *launches);

/* No counterpart in the reference.  Extraction for callers that must not
 * allocate: callbacks of a framework that owns the whole device memory pool
 * (an allocation would compete with it), or real-time loops that must never
 * block in an allocator.  It does what
 * mesh_extract_device does -- classify, scan, emit, asynchronously on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) -- but calls no
 * allocating routine: the scratch it needs lives in one static device array of
 * MESH_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits.  `vol`, `verts`, `faces` and `counts` are device memory
 * owned by the caller; counts (int64[3]) receives nverts, nfaces and the
 * device error bits (0 = complete; non-zero = outputs beyond verts_cap /
 * faces_cap were not written).  Marching Cubes reserves room for verts_cap/3
 * active cells, so its scratch grows with verts_cap; a call that needs more
 * scratch than the limit returns MESH_ESCRATCH before any GPU work.  The first
 * call on a device looks up the array's device address (once per device, kept
 * for the process: after a cudaDeviceReset of that device, do not call it on
 * that device again); make that first call before any stream capture.  All
 * calls share the array
 * and it keeps the last call's contents (each call clears what must start at
 * zero), so calls that overlap on the GPU race: serialise them. */
#define MESH_NOALLOC_SCRATCH_BYTES (64ull << 20)
MESH_API int mesh_extract_noalloc(const void *vol, int vol_dtype, int64_t nx, int64_t ny, int64_t nz,
                                  const mesh_params *p, void *verts, int64_t verts_cap, int64_t *faces,
                                  int64_t faces_cap, int64_t *counts, void *stream);

/* ---- Batches: Marching Cubes over many device volumes in one pass ----------
 * No counterpart in the reference, which extracts one volume per call
 * (src/marching_cubes.jl:27-64); each volume of a batch gives exactly what
 * that call gives on it alone.  The stages run once over a flattened worklist
 * of all volumes' tiles, with one scan across the batch, instead of one launch
 * sequence per volume.  Work is queued on the context's stream. */
typedef struct mesh_batch mesh_batch;
/* n volumes of dtype `vol_dtype` in device memory (Julia layout), vols[i] with
 * sizes dims[3i..3i+2], extracted with the MarchingCubes parameters p
 * (p->alg MESH_ALG_MC, or MESH_ALG_MC_WELDED for every volume's welded mesh:
 * the per-cell meshes are welded with edge keys made distinct per volume, and
 * the outputs, faces and rows below are the welded ones).  ranges: n x 6 endpoints (x0 x1 y0 y1 z0 z1,
 * of p->range_type), or NULL for p->range on every volume.  Pointers and sizes
 * are fixed for the batch's lifetime; the volumes' contents may change. */
MESH_API int mesh_batch_create(mesh_ctx *ctx, int n, const void *const *vols, int vol_dtype, const int64_t *dims,
                               const mesh_params *p, const double *ranges, mesh_batch **out);
MESH_API void mesh_batch_destroy(mesh_batch *b);
/* Classifies and scans every volume (waits for the result) and sizes the
 * batch's outputs exactly: total vertices and faces.  Welded batches run the
 * whole extraction and weld once here, so that the welded vertices are sized
 * exactly as well; later runs on changed contents report their welded rows in
 * the offsets. */
MESH_API int mesh_batch_count(mesh_batch *b, int64_t *nverts, int64_t *nfaces);
/* Queues the whole extraction into the batch's outputs; with graphs enabled it
 * is captured once into a CUDA graph and replayed.  Outputs larger than at the
 * last count are reported by mesh_batch_sync as MESH_ECAPACITY. */
MESH_API int mesh_batch_run(mesh_batch *b);
/* Waits for the batch's work and reports device-side errors. */
MESH_API int mesh_batch_sync(mesh_batch *b);
/* Device pointers of the outputs: vertices [V][3] of float(FT), faces [F][3]
 * int64, 1-based within each volume, and offsets [n+1][2]: the first vertex
 * and first face of volume i (row n holds the totals). */
MESH_API int mesh_batch_outputs(mesh_batch *b, void **verts, int64_t **faces, int64_t **offsets);
MESH_API int mesh_batch_set_graph(mesh_batch *b, int enable);
/* knobs[4]: z cells per work item (0 = whole columns; rounded up to 8),
 * classify and compact CTAs per SM (0 = as many as fit), threads per scan CTA
 * (96..1024, a multiple of 32).  A new first knob needs a new count. */
MESH_API int mesh_batch_set_knobs(mesh_batch *b, const int *knobs);
MESH_API int mesh_batch_knobs(const mesh_batch *b, int *knobs);
/* Autotuner: times `reps` runs of every candidate of one knob at a time,
 * keeps the fastest, counts again; a text report goes to report[report_len]. */
MESH_API int mesh_batch_tune(mesh_batch *b, int reps, char *report, int report_len);

/* ---- Serving: continuous batching of extraction requests -------------------
 * No counterpart in the reference.  Requests name a volume (device or host
 * memory) and the algorithm parameters (any of the three algorithms, welded
 * Marching Cubes included, any supported types) and are answered with exactly
 * the mesh isosurface() gives for them alone.
 * A loop thread admits queued requests in arrival order into waves whenever a
 * slot is free and the device pool (budget_bytes, allocated at creation) can
 * reserve each request's worst-case output: 12 vertices and 5 faces per cell
 * for Marching Cubes, 7 vertices per node and 12 faces per cell for Marching
 * Tetrahedra, 1 vertex per cell and 6 faces per node for Naive Surface Nets.
 * Marching Cubes requests of a wave with the same volume type and iso run as
 * one batch; waves on different slots overlap on the device.  A request's mesh
 * stays resident in the pool until mesh_server_release.  Thread-safe.
 * slots (1..16): waves in flight at once, each capped at budget_bytes / slots
 * beyond its first request; max_wave: requests per wave; max_queue: waiting
 * requests beyond which mesh_server_submit rejects (MESH_EBUSY). */
typedef struct mesh_server mesh_server;
MESH_API int mesh_server_create(int device, int64_t budget_bytes, int slots, int max_wave, int max_queue,
                                mesh_server **out);
/* Stops admitting, waits for the waves in flight, frees the pool. */
MESH_API void mesh_server_destroy(mesh_server *s);
MESH_API const char *mesh_server_last_error(const mesh_server *s);
/* Queues a request; *id identifies it.  vol_on_device = 0: vol is host memory
 * (pinned uploads fastest), copied into the pool when the request is admitted
 * to a wave -- it must stay valid and unchanged until the request has ended;
 * its bytes count against the budget like the outputs while the request is in
 * flight.  MESH_EBUDGET: its worst case alone exceeds the budget; MESH_EBUSY:
 * max_queue requests are waiting.  Welded Marching Cubes requests also use the
 * slot context's own scratch for the mesh before welding. */
MESH_API int mesh_server_submit(mesh_server *s, const void *vol, int vol_dtype, int64_t nx, int64_t ny, int64_t nz,
                                int vol_on_device, const mesh_params *p, int64_t *id);
/* state: 0 queued, 1 running, 2 done, 3 failed (the return value is then the
 * failure's status).  When done: counts and device pointers of the vertices
 * (float(FT) triples) and faces (1-based int64 triples). */
MESH_API int mesh_server_poll(mesh_server *s, int64_t id, int *state, int64_t *nverts, int64_t *nfaces,
                              void **verts, int64_t **faces);
/* As mesh_server_poll after waiting up to timeout_us for the request to end. */
MESH_API int mesh_server_wait(mesh_server *s, int64_t id, int64_t timeout_us, int *state, int64_t *nverts,
                              int64_t *nfaces, void **verts, int64_t **faces);
/* Frees a finished request's output block (its pointers become invalid). */
MESH_API int mesh_server_release(mesh_server *s, int64_t id);
/* stats[14]: completed, rejected, failed, p50 / p99 / mean latency in ms
 * (submission to completion on the device), input samples completed, seconds
 * from the first submission to the last completion, peak / capacity pool
 * bytes, queued requests, currently reserved pool bytes, waves launched,
 * requests per wave.  A finished request keeps only its mesh reserved. */
MESH_API int mesh_server_stats(mesh_server *s, double *stats);
MESH_API int mesh_server_reset_stats(mesh_server *s);
/* Load generator for measurements: submits request i (vols[i] of dtypes[i],
 * sizes dims[3i..3i+2], params[i]) arrivals_s[i] seconds after the call
 * starts, releases each request as soon as it ends, and returns when all have
 * ended.  Rejected submissions count in the stats. */
MESH_API int mesh_server_replay(mesh_server *s, int n, const void *const *vols, const int *dtypes,
                                const int64_t *dims, const mesh_params *params, const double *arrivals_s);

#ifdef __cplusplus
}
#endif
#endif /* MESHING_GB300_H */
