// Host-side state shared by the single-volume runtime (mesh_api.cu) and the
// batched runtime (mesh_batch.cu).  Not part of the public ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "mesh_internal.cuh"

namespace mesh {

constexpr int NSTAGE = 4;  // classify (or the one-walk MC pass), scan, emit (second walk), expand
// device word slots of the misc buffer: totals[NCNT], error word, work counter,
// staging counter
constexpr int MISC_SLOTS = NCNT + 3;
// parts of the pipelined host path: upload groups of z segments, x ranges of the emission
constexpr int PIPE_MAX = 8;

struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap) return cudaSuccess;
        size_t want = std::max(n, cap + cap / 4);
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            e = cudaMalloc(&ptr, n);
            if (e != cudaSuccess) return e;
            want = n;
        }
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
    }
};

}  // namespace

struct mesh_ctx {
    int device = 0;
    int sms = 148;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    mesh::DevBuf vol, tabs, cnt, base, flags, scan, misc, out_v, out_f, ent;
    mesh::DevBuf nrm;  // mesh_vertex_normals: double accumulators
    mesh::DevBuf cmask;  // Marching Cubes: per (x tile, cell row, chunk) active-column masks
    // welded Marching Cubes (MESH_ALG_MC_WELDED): the count runs the whole
    // extraction into out_v / out_f and welds it into weld_v; mesh_fill copies
    int weld = 0;
    mesh::DevBuf weld_buf, weld_v;
    int64_t *h_misc = nullptr;  // pinned: totals[NCNT], err
    // Pipelined host path (MESHING_GB300_PIPELINE_BYTES, default 256 MiB: host
    // volumes and meshes at least this large).  mesh_count uploads the volume in
    // groups of z segments on the copy stream and classifies each group as soon
    // as its planes have arrived; mesh_fill emits the Marching Cubes mesh in x
    // ranges (contiguous in the x-major emission order) and downloads each range
    // on the copy stream while the next one is emitted.  Events order the two
    // streams; the split points come from the scanned piece bases (gat / h_gat).
    int64_t pipe_bytes = (int64_t)256 << 20;
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_ready = nullptr, ev_done = nullptr;
    cudaEvent_t ev_part[mesh::PIPE_MAX] = {};
    int ngroups = 1;
    const void *upl_src = nullptr;  // the host volume of the count in progress
    mesh::DevBuf gat;
    int64_t *h_gat = nullptr;
    mesh::Plan plan{};
    int have_plan = 0;
    int Q64 = 0, A64 = 0, P64 = 0;
    int64_t nverts = 0, nfaces = 0, nactive = 0;
    int64_t ent_cap_seen = 0;  // largest active-cell list prepared on this context
    // mesh_set_x_window: the volumes of the following calls are x nodes
    // win_x0 .. win_x0+nx-1 of an x axis of win_nx nodes (win_nx == 0: whole axis)
    int64_t win_x0 = 0, win_nx = 0;
    int win_halo = 0;  // MT / NSN: the first cell column is the previous slab's last one
    std::string msg;
    // stage timing (diagnostics)
    int timing = 0;
    int force_fp64 = 0;  // MESHING_GB300_FORCE_FP64=1: evaluate every Float64 position in FP64
    // Classification from TMA-staged bricks: by default for Marching Cubes volumes a
    // tensor map can describe (Float32 / UInt16 / Float64, 16-byte row strides) and
    // not uploaded in pipelined groups; MESHING_GB300_TMA=0 (-1 unset) keeps the
    // global-load walk, MESHING_GB300_TMA=1 also streams MT / NSN volumes.
    int tma_env = -1;
    // MESHING_GB300_ONE_WALK=1: Marching Cubes in one walk that also lists the
    // active cells (k_walk_mc.cu).  Off by default: on GB300 the walk is issue
    // bound, so dropping the second read of the volume saves little, and
    // expanding the cells in walk order scatters the output writes (1024^3 f32:
    // walk 2.24 + expand 1.41 ms vs classify 1.24 + compact 1.18 + expand 0.75 ms).
    int one_walk = 0;
    // MESHING_GB300_LIST_EMIT=1: Marching Cubes emitted through the list of
    // active cells (compaction, then expansion) instead of straight from the
    // volume (k_direct_mc.cu); kept for comparison tests.
    int list_emit = 0;
    // MESHING_GB300_ZEROCOPY=1: a Marching Cubes host volume in pinned, mapped
    // memory is read in place over the host link (NVLink-C2C) by the one walk
    // instead of being copied.  Off by default: on GB300 the in-place walk of a
    // 4 GiB volume ran at the link's ~140 GB/s, no faster than the copy, and the
    // one-walk expansion costs more (end to end 42.1 vs 33.6 ms at 1024^3).
    int zerocopy = 0;
    int host_mapped = 0; // the current plan reads a mapped host volume
    int use_tma = 0;     // the current plan streams the volume through TMA
    CUtensorMap tmap;
    std::vector<cudaEvent_t> ev_free;
    std::vector<cudaEvent_t> ev_pairs[mesh::NSTAGE];  // start, stop, start, stop, ...
    int64_t nkern[mesh::NSTAGE] = {};                 // kernels launched per stage (with timing on)
};

namespace mesh {

// Error helpers: record a message on the context and return the status.
int fail(mesh_ctx *c, int status, const char *fmt, ...);
int cuda_fail(mesh_ctx *c, cudaError_t e, const char *what);
// Argument checks shared by every entry point.
int validate(mesh_ctx *c, int T, int64_t nx, int64_t ny, int64_t nz, const mesh_params *p);
// Julia's promotion: arithmetic types (Q64: quotient in Float64, A64: MT clamp in
// Float64, P64: positions in Float64), output eltype and the exact thresholds.
void set_types(Plan &P, int T, const mesh_params *p, int *Q64, int *A64, int *P64);

// Tiling of a batch of volumes of sizes dims[3i..3i+2] with `zs` z cells per
// work item (0 = whole columns): the descriptors (without device pointers),
// each volume's table block offset in doubles, and the totals.
struct BatchSizes {
    int64_t items = 0, pieces = 0, nflags = 0, tdoubles = 0, stiles = 0, max_ntab = 1;
    int64_t keys = 0;  // lattice-edge keys of all volumes (3 per node)
};
BatchSizes tile_batch(const int64_t *dims, int n, int zs, std::vector<BatchVol> &hv, std::vector<int64_t> &tab_off);
// The volume of every work item and scan tile.
void batch_owners(const std::vector<BatchVol> &hv, const BatchSizes &z, std::vector<uint32_t> &ivol,
                  std::vector<uint32_t> &svol);

}  // namespace mesh
