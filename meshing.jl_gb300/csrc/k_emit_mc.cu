// K3 (Marching Cubes), two-pass form -- emit vertices and faces at the
// scanned offsets, after a second walk over the volume.
//
// Replaces process_mc_voxel! (src/marching_cubes.jl:67-92).  Two kernels:
//
// K3a compact.  Persistent warps walk the classify kernel's tiles (31 x-cells
// by WY y-cells, one z segment), skipping z chunks whose activity bytes are
// zero and z steps whose corners all lie on one side of iso.  Every active
// cell gets one entry -- packed (x, y, z), case, its 8 corner values -- at
// index base_a(piece) + running count, i.e. the list of active cells in the
// reference's emission order.  Every 256th entry also records the global
// vertex and face offsets of its cell.
//
// K3b expand (mesh_mc.cuh, k_expand_mc<..., EXP_ORDERED>).
//
// This is the default form: the one walk of k_walk_mc.cu reads the volume
// once but costs more in total on GB300.  Its scratch is also known exactly
// after the scan, which the allocation-free entry point needs.
#define MESH_TBL static __device__ const
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_mc.cuh"

#include <algorithm>

namespace mesh {

namespace {

constexpr int U = 4;     // z planes loaded ahead (only active chunks are walked)
// A chunk's last loaded plane becomes the next chunk's first (lov = v[U-1]), so a
// group of U planes must never straddle a chunk boundary.
static_assert(ZC % U == 0, "U must divide the activity chunk");

// ---------------------------------------------------------------- K3a ----

// Entries of warp tile (tx, ty) of z segment seg; with a batch, each entry
// also records its volume `vol`.
template <class T>
__device__ __forceinline__ void compact_tile(const Plan &p, const uint64_t *s_v, int lane, int tx, int ty, int seg,
                                             uint32_t vol) {
    const T *volp = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;
    const int64_t np = p.pstride;
    {
        const int xs = tx * TILE_X + lane;
        const int y0 = ty * WY;
        const int zbeg = seg * p.zs;
        const int zend = min(zbeg + p.zs, p.cz);
        const bool cellx = lane < TILE_X && xs < p.cx;

        bool rowok[WY + 1];
        const T *rowp[WY + 1];
#pragma unroll
        for (int r = 0; r <= WY; r++) {
            rowok[r] = xs < p.nx && y0 + r < p.ny;
            rowp[r] = rowok[r] ? volp + xs + p.nx * (int64_t)(y0 + r) : volp;
        }
        const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
        const uint32_t cellm = __ballot_sync(FULL, cellx);
        int64_t bv[WY], bf[WY], ba[WY];  // running vertex / face / entry offsets of each row's cell
#pragma unroll
        for (int r = 0; r < WY; r++) {
            bv[r] = bf[r] = ba[r] = 0;
            if (cellx && y0 + r < p.cy) {
                const int64_t i = piece(p, seg, y0 + r, xs);
                bv[r] = p.base[i];
                bf[r] = p.base[np + i];
                ba[r] = p.base[2 * np + i];
            }
        }

        uint32_t mlo[WY + 1];
        T lov[WY + 1];  // samples of plane z
        bool have_lo = false;
        for (int zc0 = zbeg; zc0 < zend; zc0 += ZC) {
            const int zc1 = min(zc0 + ZC, zend);
            const int chunk = seg * p.chunks_per_seg + (zc0 - zbeg) / ZC;
            uint8_t f = 0;
            if (lane < WY && y0 + lane < p.cy) f = p.flags[((int64_t)chunk * p.tiles_x + tx) * p.cy + y0 + lane];
            if (!__any_sync(FULL, f != 0)) {
                have_lo = false;
                continue;
            }
            if (!have_lo) {
#pragma unroll
                for (int r = 0; r <= WY; r++) {
                    lov[r] = rowok[r] ? ldv(rowp[r] + sxy * (int64_t)zc0) : T(0);
                    mlo[r] = __ballot_sync(FULL, rowok[r] && below(lov[r], p));
                }
                have_lo = true;
            }
            for (int z = zc0; z < zc1; z += U) {
                T v[U][WY + 1];
                const int64_t off = sxy * (int64_t)(z + 1);
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int r = 0; r <= WY; r++)
                        v[u][r] = (rowok[r] && z + 1 + u <= zc1) ? ldv(rowp[r] + off + sxy * u) : T(0);
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int zc = z + u;
                    if (zc >= zc1) break;
                    uint32_t mhi[WY + 1];
                    uint32_t all1 = xval, any1 = 0;
#pragma unroll
                    for (int r = 0; r <= WY; r++) {
                        mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
                        all1 &= mlo[r] & mhi[r];
                        any1 |= mlo[r] | mhi[r];
                    }
                    if (all1 != xval && any1 != 0) {
#pragma unroll
                        for (int r = 0; r < WY; r++) {
                            const uint32_t and4 = mlo[r] & mlo[r + 1] & mhi[r] & mhi[r + 1];
                            const uint32_t or4 = mlo[r] | mlo[r + 1] | mhi[r] | mhi[r + 1];
                            const uint32_t actm = (or4 | (or4 >> 1)) & ~(and4 & (and4 >> 1)) & cellm;
                            if (actm == 0u || y0 + r >= p.cy) continue;  // warp-uniform
                            // corner values; x+1 from the next lane
                            const T a0 = u == 0 ? lov[r] : v[u == 0 ? 0 : u - 1][r];
                            const T b0 = u == 0 ? lov[r + 1] : v[u == 0 ? 0 : u - 1][r + 1];
                            const T c0 = v[u][r], d0 = v[u][r + 1];
                            const T a1 = shfl_down1(a0), b1 = shfl_down1(b0), c1 = shfl_down1(c0), d1 = shfl_down1(d0);
                            if ((actm >> lane) & 1u) {
                                const unsigned a = (mlo[r] >> lane) & 3u, b = (mlo[r + 1] >> lane) & 3u;
                                const unsigned c = (mhi[r] >> lane) & 3u, d = (mhi[r + 1] >> lane) & 3u;
                                const unsigned cm = (a & 1u) | ((a >> 1) << 1) | ((b >> 1) << 2) | ((b & 1u) << 3) |
                                                    ((c & 1u) << 4) | ((c >> 1) << 5) | ((d >> 1) << 6) |
                                                    ((d & 1u) << 7);
                                const int64_t e = ba[r];
                                if (e < p.ent_cap) {
                                    p.ent_pos[e] = (unsigned long long)xs |
                                                   ((unsigned long long)(y0 + r) << POS_BITS) |
                                                   ((unsigned long long)zc << (2 * POS_BITS));
                                    p.ent_cs[e] = (uint8_t)cm;
                                    const T cv[8] = {a0, a1, b1, b0, c0, c1, d1, d0};
                                    store8<T>((T *)p.ent_val + 8 * e, cv);
                                    if (p.ent_vol) p.ent_vol[e] = vol;
                                    if ((e & (ENT_BLOCK - 1)) == 0) {
                                        p.ent_side[2 * (e / ENT_BLOCK)] = bv[r];
                                        p.ent_side[2 * (e / ENT_BLOCK) + 1] = bf[r];
                                    }
                                } else {
                                    atomicOr(p.err, ERR_CAPACITY);
                                }
                                const uint64_t t = s_v[cm];
                                ba[r] = e + 1;
                                bv[r] += (int64_t)((t >> 48) & 15u);
                                bf[r] += (int64_t)((t >> 52) & 7u);
                            }
                        }
                    }
#pragma unroll
                    for (int r = 0; r <= WY; r++) mlo[r] = mhi[r];
                }
#pragma unroll
                for (int r = 0; r <= WY; r++) lov[r] = v[U - 1][r];
            }
        }
    }
}

template <class T>
__global__ void __launch_bounds__(256, 2) k_compact_mc(const Plan p, int nitems) {
    __shared__ uint64_t s_v[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_v[i] = MC_CASE_VERTS[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    // persistent warps: take (y tile, x tile, segment) items in order from a counter
    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nitems) break;
        const int ty = item % p.tiles_y;
        const int tx = (item / p.tiles_y) % p.tiles_x;
        const int seg = item / (p.tiles_y * p.tiles_x);
        compact_tile<T>(p, s_v, lane, tx, ty, seg, 0);
    }
}

// Batch: the work items of k_classify_batch, in the same order.
template <class T>
__global__ void __launch_bounds__(256, 2) k_compact_batch(const Plan p) {
    __shared__ uint64_t s_v[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_v[i] = MC_CASE_VERTS[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned item = 0;
        if (lane == 0) item = atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if ((int64_t)item >= p.nitems) break;
        const uint32_t v = p.item_vol[item];
        const BatchVol b = p.bvols[v];
        const int64_t local = (int64_t)item - b.item0;
        const int ty = (int)(local % b.tiles_y);
        const int tx = (int)((local / b.tiles_y) % b.tiles_x);
        const int seg = (int)(local / ((int64_t)b.tiles_y * b.tiles_x));
        compact_tile<T>(vol_view(p, b), s_v, lane, tx, ty, seg, v);
    }
}

template <class T, class Q, class P> cudaError_t go(const Plan &p, int stage, cudaStream_t s) {
    static int grid_a = 0, grid_b = 0;  // per instantiation: resident CTAs on this device
    if (!grid_a) {
        grid_a = resident_ctas((const void *)k_compact_mc<T>, 32 * WARPS);
        grid_b = resident_ctas((const void *)k_expand_mc<T, Q, P, EXP_ORDERED>, XW);
    }
    if (stage == 0) {
        const int nitems = p.tiles_x * p.tiles_y * p.nseg;
        cudaError_t e = cudaMemsetAsync(p.work, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
        k_compact_mc<T><<<std::min(grid_a, (nitems + WARPS - 1) / WARPS), 32 * WARPS, 0, s>>>(p, nitems);
    } else {
        k_expand_mc<T, Q, P, EXP_ORDERED><<<grid_b, XW, 0, s>>>(p);
    }
    return cudaGetLastError();
}

template <class T> cudaError_t go_t(const Plan &p, int Q64, int P64, int stage, cudaStream_t s) {
    if (Q64) return go<T, double, double>(p, stage, s);
    if (P64) return go<T, float, double>(p, stage, s);
    return go<T, float, float>(p, stage, s);
}

int persistent_ctas(const void *fn, int threads, int ctas_per_sm) {
    int dev = 0, sms = 0, fit = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, fn, threads, 0) != cudaSuccess || fit < 1) {
        cudaGetLastError();
        fit = 1;
    }
    return sms * (ctas_per_sm > 0 ? std::min(ctas_per_sm, fit) : fit);
}

template <class T> cudaError_t compact_batch_t(const Plan &p, int ctas, cudaStream_t s) {
    const int grid = (int)std::min<int64_t>(persistent_ctas((const void *)k_compact_batch<T>, 32 * WARPS, ctas),
                                            (p.nitems + WARPS - 1) / WARPS);
    cudaError_t e = cudaMemsetAsync(p.work, 0, sizeof(unsigned), s);
    if (e != cudaSuccess || grid < 1) return e;
    k_compact_batch<T><<<grid, 32 * WARPS, 0, s>>>(p);
    return cudaGetLastError();
}

template <class T, class Q, class P> cudaError_t expand_batch_t(const Plan &p, cudaStream_t s) {
    static int grid = 0;  // per instantiation: resident CTAs on this device
    if (!grid) grid = resident_ctas((const void *)k_expand_mc<T, Q, P, EXP_BATCH>, XW);
    k_expand_mc<T, Q, P, EXP_BATCH><<<grid, XW, 0, s>>>(p);
    return cudaGetLastError();
}

template <class T> cudaError_t expand_batch_tt(const Plan &p, int Q64, int P64, cudaStream_t s) {
    if (Q64) return expand_batch_t<T, double, double>(p, s);
    if (P64) return expand_batch_t<T, float, double>(p, s);
    return expand_batch_t<T, float, float>(p, s);
}

}  // namespace

cudaError_t launch_compact_batch(const Plan &p, int ctas, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return compact_batch_t<uint16_t>(p, ctas, s);
    case MESH_DT_F32: return compact_batch_t<float>(p, ctas, s);
    case MESH_DT_I32: return compact_batch_t<int32_t>(p, ctas, s);
    case MESH_DT_I64: return compact_batch_t<int64_t>(p, ctas, s);
    default: return compact_batch_t<double>(p, ctas, s);
    }
}

cudaError_t launch_expand_batch(const Plan &p, int Q64, int P64, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return expand_batch_tt<uint16_t>(p, Q64, P64, s);
    case MESH_DT_F32: return expand_batch_tt<float>(p, Q64, P64, s);
    case MESH_DT_I32: return expand_batch_tt<int32_t>(p, Q64, P64, s);
    case MESH_DT_I64: return expand_batch_tt<int64_t>(p, Q64, P64, s);
    default: return expand_batch_t<double, double, double>(p, s);
    }
}

// stage 0: K3a compact (active-cell list); stage 1: K3b expand (vertices and faces)
cudaError_t launch_emit_mc(const Plan &p, int Q64, int P64, int stage, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return go_t<uint16_t>(p, Q64, P64, stage, s);
    case MESH_DT_F32: return go_t<float>(p, Q64, P64, stage, s);
    case MESH_DT_I32: return go_t<int32_t>(p, Q64, P64, stage, s);
    case MESH_DT_I64: return go_t<int64_t>(p, Q64, P64, stage, s);
    default: return go<double, double, double>(p, stage, s);
    }
}

}  // namespace mesh
