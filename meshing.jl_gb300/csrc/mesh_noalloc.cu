// mesh_extract_noalloc: isosurface extraction that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they extract a
// mesh: callbacks of a host framework that owns the whole device memory pool
// (an allocation would compete with it), or real-time loops that must never
// block in the allocator.  This entry point serves them.  The caller passes the volume, the output buffers
// and a small counts buffer (device memory it already owns); every piece of
// scratch the kernels need -- per-column counts and their scan, activity
// bytes, look-back state, coordinate tables, the Marching Cubes active-cell
// list -- lives in one file-scope __device__ array of NOALLOC_SCRATCH_BYTES.
// The coordinate tables are computed on the device with the same arithmetic
// the host path uses, so no host buffer is needed either.
//
// The array belongs to the module: every GPU that loads this library holds
// it until the process exits.  All calls on a device share it and it keeps
// the last call's contents; everything that must start at zero is cleared at
// the start of each call.  Calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the array and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "mesh_internal.cuh"
#include "mesh_tables.h"

namespace mesh {
cudaError_t launch_emit_mc(const Plan &p, int Q64, int P64, int stage, cudaStream_t s);
cudaError_t launch_emit_halo(const Plan &p, int Q64, int A64, int P64, cudaStream_t s);
size_t scan_scratch_bytes(const Plan &p);
void set_types(Plan &P, int T, const mesh_params *p, int *Q64, int *A64, int *P64);
}  // namespace mesh

using namespace mesh;

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = MESH_NOALLOC_SCRATCH_BYTES;  // 64 MiB

static __device__ __align__(256) unsigned char g_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
void *g_scratch_ptr[MAX_DEVICES];  // device address of g_scratch, per device
std::mutex g_setup;

// The device address of g_scratch on the current device; looked up once per
// device and kept for the process (host code cannot use the symbol itself as
// an address).  A cudaDeviceReset loads the module again, possibly elsewhere:
// the header tells callers not to use this entry point on a device after that.
cudaError_t scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

size_t up256(size_t n) { return (n + 255) / 256 * 256; }

}  // namespace

extern "C" int mesh_extract_noalloc(const void *vol, int T, int64_t nx, int64_t ny, int64_t nz,
                                             const mesh_params *prm, void *verts, int64_t verts_cap, int64_t *faces,
                                             int64_t faces_cap, int64_t *counts, void *stream_handle) {
    if (!prm || !counts) return MESH_EINVAL;
    if (prm->alg == MESH_ALG_MC_WELDED) return MESH_EINVAL;  // welding needs scratch of its own
    int bits = 0;
    int rc = mesh_output_float_bits(T, prm, &bits);  // validates types and values
    if (rc) return rc;
    const int64_t lim = (int64_t)1 << POS_BITS;
    if (nx < 0 || ny < 0 || nz < 0) return MESH_EINVAL;
    if (nx > lim || ny > lim || nz > lim) return MESH_ETOOLARGE;
    cudaStream_t s = (cudaStream_t)stream_handle;
    cudaError_t e;
    if ((e = cudaMemsetAsync(counts, 0, 3 * sizeof(int64_t), s)) != cudaSuccess) return MESH_ECUDA;
    if (nx < 2 || ny < 2 || nz < 2) return MESH_OK;
    if (!vol || (verts_cap > 0 && !verts) || (faces_cap > 0 && !faces)) return MESH_EINVAL;

    Plan P{};
    P.vol = vol;
    P.nx = nx; P.ny = ny; P.nz = nz;
    P.cx = (int32_t)(nx - 1); P.cy = (int32_t)(ny - 1); P.cz = (int32_t)(nz - 1);
    // types, thresholds and MT clamps exactly as the context path sets them
    int Q64 = 0, A64 = 0, P64 = 0;
    set_types(P, T, prm, &Q64, &A64, &P64);
    const int L32 = prm->range_type == MESH_DT_F32;
    if (P.out64 != (bits == 64)) return MESH_EINVAL;
    // one z segment per column keeps the per-piece scratch small
    P.tiles_x = (P.cx + TILE_X - 1) / TILE_X;
    P.tiles_y = (P.cy + WY - 1) / WY;
    P.zs = (P.cz + ZC - 1) / ZC * ZC;
    P.nseg = 1;
    P.chunks_per_seg = P.zs / ZC;
    P.nchunks = P.chunks_per_seg;
    if ((P.tiles_y + WARPS - 1) / WARPS > 65535) return MESH_ETOOLARGE;

    // scratch layout inside g_scratch (each array 256-byte aligned)
    const int64_t ntab = nx + ny + nz;
    const int64_t np = npieces(P);
    const size_t sb = (scan_scratch_bytes(P) + 255) / 256 * 256;
    const size_t es = dtype_size(T);
    const int64_t cap = prm->alg == MESH_ALG_MC ? verts_cap / 3 : 0;  // active MC cells emit >= 3 vertices
    const int64_t nside = cap / ENT_BLOCK + 1;
    size_t off = 0;
    const size_t o_misc = off;   off += up256((NCNT + 2) * sizeof(int64_t));
    const size_t o_scan = off;   off += up256(sb + 64);
    const size_t o_tab = off;    off += up256(table_bytes(ntab));
    const size_t o_cnt = off;    off += up256((size_t)np * NCNT * 4);
    const size_t o_base = off;   off += up256((size_t)np * NCNT * 8);
    const size_t o_flags = off;  off += up256((size_t)P.nchunks * P.tiles_x * P.cy);
    const size_t o_pos = off;    off += up256((size_t)cap * 8);
    const size_t o_val = off;    off += up256((size_t)cap * 8 * es);
    const size_t o_side = off;   off += up256((size_t)nside * 16);
    const size_t o_cs = off;     off += up256((size_t)cap + 1);
    if (off > NOALLOC_SCRATCH_BYTES) return MESH_ESCRATCH;

    unsigned char *base = nullptr;
    if ((e = scratch_address((void **)&base)) != cudaSuccess) return MESH_ECUDA;
    P.totals = (int64_t *)(base + o_misc);
    P.err = (unsigned int *)((int64_t *)(base + o_misc) + NCNT);
    P.work = (unsigned int *)((int64_t *)(base + o_misc) + NCNT + 1);
    P.scan_state = (unsigned long long *)(base + o_scan);
    P.scan_ticket = (unsigned int *)(base + o_scan + sb);
    double *dp = (double *)(base + o_tab);
    bind_tables(P, dp, nx, ny, nz);
    P.pstride = np;
    P.cnt = (uint32_t *)(base + o_cnt);
    P.base = (int64_t *)(base + o_base);
    P.flags = base + o_flags;
    P.ent_pos = (unsigned long long *)(base + o_pos);
    P.ent_val = base + o_val;
    P.ent_side = (long long *)(base + o_side);
    P.ent_cs = base + o_cs;
    P.ent_cap = cap;
    P.verts = verts;
    P.faces = faces;
    P.verts_cap = verts ? verts_cap : 0;
    P.faces_cap = faces ? faces_cap : 0;
    P.scan_spin_limit = 1 << 24;

    // totals, error word and work counter start at zero; the rest is overwritten
    if ((e = cudaMemsetAsync(base + o_misc, 0, (NCNT + 2) * sizeof(int64_t), s)) != cudaSuccess) return MESH_ECUDA;
    if ((e = launch_tables(dp, nx, ny, nz, prm->range, L32, s)) != cudaSuccess) return MESH_ECUDA;
    if ((e = launch_classify(P, s)) != cudaSuccess) return MESH_ECUDA;
    if ((e = launch_scan(P, s)) != cudaSuccess) return MESH_ECUDA;
    if (P.alg == MESH_ALG_MC) {
        e = launch_emit_mc(P, Q64, P64, 0, s);
        if (e == cudaSuccess) e = launch_emit_mc(P, Q64, P64, 1, s);
    } else {
        e = launch_emit_halo(P, Q64, A64, P64, s);
    }
    if (e != cudaSuccess) return MESH_ECUDA;
    // counts[0..1] = totals; counts[2] = device error bits (0 when the outputs are complete)
    if ((e = cudaMemcpyAsync(counts, P.totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return MESH_ECUDA;
    if ((e = cudaMemcpyAsync(counts + 2, P.err, sizeof(unsigned int), cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return MESH_ECUDA;
    return MESH_OK;
}
