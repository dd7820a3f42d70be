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
#include "mesh_case.cuh"
#include "mesh_mc.cuh"

#include <algorithm>
#include <mutex>

namespace mesh {

namespace {

constexpr int U = 8;     // z planes loaded ahead (only active chunks are walked)
// A chunk's last loaded plane becomes the next chunk's first (lov = v[U-1]), so a
// group of U planes must never straddle a chunk boundary.
static_assert(ZC % U == 0, "U must divide the activity chunk");

// ---------------------------------------------------------------- K3a ----

// Shared memory of a compaction CTA: the case tables and, per warp, the
// global vertex / face offsets of the lanes' pieces (needed only at chunk ends
// and for the side words, so they stay out of registers).
struct CompactSmem {
    uint32_t pk[256];
    uint8_t cs[256];
    long long bv[WARPS][WY][32], bf[WARPS][WY][32];
};

// Entries of warp tile (tx, ty) of z segment seg; with a batch, each entry
// also records its volume `vol`.  The activity bytes of 32 chunks are read at
// once and the walk visits only the active chunks.  Inside a chunk a step whose corners are not all on one side costs,
// per cell row, one lookup of the case's packed word (mesh_case.cuh); the
// lanes whose cell is active write its entry at the piece's entry offset plus
// the entries before it in the chunk (bits 23.. of the running word).
template <class T, int NR>
__device__ __forceinline__ void compact_tile(const Plan &p, CompactSmem &sm, int w, int lane, int tx, int ty, int seg,
                                             uint32_t vol) {
    const T *volp = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;
    const int64_t np = p.pstride;
    const int xs = tx * TILE_X + lane;
    const int y0 = ty * NR;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < TILE_X && xs < p.cx;

    bool rowok[NR + 1];
    const T *rowp[NR + 1];
#pragma unroll
    for (int r = 0; r <= NR; r++) {
        rowok[r] = xs < p.nx && y0 + r < p.ny;
        rowp[r] = rowok[r] ? volp + xs + p.nx * (int64_t)(y0 + r) : volp;
    }
    const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
    uint32_t rmask[NR];
    int64_t ba[NR];  // entry offset of each row's piece
#pragma unroll
    for (int r = 0; r < NR; r++) {
        rmask[r] = (cellx && y0 + r < p.cy) ? 0xffffffffu : 0u;
        ba[r] = 0;
        long long v0 = 0, f0 = 0;
        if (rmask[r]) {
            const int64_t i = piece(p, seg, y0 + r, xs);
            v0 = p.base[i];
            f0 = p.base[np + i];
            ba[r] = p.base[2 * np + i];
        }
        sm.bv[w][r][lane] = v0;
        sm.bf[w][r][lane] = f0;
    }
    __syncwarp();

    // activity of chunks [32 g, 32 g + 32): lane l reads chunk 32 g + l's row bytes
    const int nch = (zend - zbeg + ZC - 1) / ZC;
    const int64_t chunk0 = (int64_t)seg * p.chunks_per_seg;
    auto active = [&](int g) {
        const int k = 32 * g + lane;
        uint32_t any = 0;
        if (k < nch) {
            const uint8_t *fp = p.flags + ((chunk0 + k) * p.tiles_x + tx) * p.cy + y0;
#pragma unroll
            for (int r = 0; r < NR; r++)
                if (y0 + r < p.cy) any |= fp[r];
        }
        return __ballot_sync(FULL, any != 0u);
    };

    uint32_t mlo[NR + 1];
    T lov[NR + 1];  // samples of plane `have`
    int have = -1;
    for (int g = 0; 32 * g < nch; g++) {
        uint32_t todo = active(g);
        while (todo) {
            const int k = __ffs(todo) - 1;
            todo &= todo - 1;
            const int zc0 = zbeg + k * ZC + 32 * g * ZC;
            const int zc1 = min(zc0 + ZC, zend);
            if (have != zc0) {
#pragma unroll
                for (int r = 0; r <= NR; r++) {
                    lov[r] = rowok[r] ? ldv(rowp[r] + sxy * (int64_t)zc0) : T(0);
                    mlo[r] = __ballot_sync(FULL, rowok[r] && below(lov[r], p));
                }
            }
            uint32_t pk[NR];
#pragma unroll
            for (int r = 0; r < NR; r++) pk[r] = 0;
            for (int z = zc0; z < zc1; z += U) {
                T v[U][NR + 1];
                const int64_t off = sxy * (int64_t)(z + 1);
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int r = 0; r <= NR; r++)
                        v[u][r] = (rowok[r] && z + 1 + u <= zc1) ? ldv(rowp[r] + off + sxy * u) : T(0);
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int zc = z + u;
                    if (zc >= zc1) break;  // warp-uniform
                    uint32_t mhi[NR + 1];
                    uint32_t all1 = xval, any1 = 0;
#pragma unroll
                    for (int r = 0; r <= NR; r++) {
                        mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
                        all1 &= mlo[r] & mhi[r];
                        any1 |= mlo[r] | mhi[r];
                    }
                    if (all1 != xval && any1 != 0u) {
                        // corner values of row r in plane z (l0) and z+1 (h0), x+1 from
                        // the next lane (l1, h1); row r+1 likewise (L0 L1 H0 H1)
                        T l0 = u == 0 ? lov[0] : v[u == 0 ? 0 : u - 1][0];
                        T h0 = v[u][0];
                        T l1 = shfl_down1(l0), h1 = shfl_down1(h0);
                        uint32_t n0 = row_field(mlo[0], mhi[0], lane);
#pragma unroll
                        for (int r = 0; r < NR; r++) {
                            const T L0 = u == 0 ? lov[r + 1] : v[u == 0 ? 0 : u - 1][r + 1];
                            const T H0 = v[u][r + 1];
                            const T L1 = shfl_down1(L0), H1 = shfl_down1(H0);
                            const uint32_t n1 = row_field(mlo[r + 1], mhi[r + 1], lane);
                            const unsigned idx = n0 | (n1 << 4);
                            const uint32_t t = sm.pk[idx] & rmask[r];
                            if (t) {
                                const int64_t e = ba[r] + (pk[r] >> PK_A);
                                if (e < p.ent_cap) {
                                    p.ent_pos[e] = (unsigned long long)xs |
                                                   ((unsigned long long)(y0 + r) << POS_BITS) |
                                                   ((unsigned long long)zc << (2 * POS_BITS));
                                    p.ent_cs[e] = sm.cs[idx];
                                    const T cv[8] = {l0, l1, L1, L0, h0, h1, H1, H0};
                                    store8<T>((T *)p.ent_val + 8 * e, cv);
                                    if (p.ent_vol) p.ent_vol[e] = vol;
                                    if ((e & (ENT_BLOCK - 1)) == 0) {
                                        p.ent_side[2 * (e / ENT_BLOCK)] =
                                            sm.bv[w][r][lane] + (pk[r] & ((1u << PK_F) - 1u));
                                        p.ent_side[2 * (e / ENT_BLOCK) + 1] =
                                            sm.bf[w][r][lane] + ((pk[r] >> PK_F) & ((1u << (PK_A - PK_F)) - 1u));
                                    }
                                } else {
                                    atomicOr(p.err, ERR_CAPACITY);
                                }
                                pk[r] += t;
                            }
                            l0 = L0;
                            l1 = L1;
                            h0 = H0;
                            h1 = H1;
                            n0 = n1;
                        }
                    }
#pragma unroll
                    for (int r = 0; r <= NR; r++) mlo[r] = mhi[r];
                }
#pragma unroll
                for (int r = 0; r <= NR; r++) lov[r] = v[U - 1][r];
            }
            // a chunk of ZC planes ends on whole groups of U (ZC % U == 0), so
            // lov / mlo hold plane zc1; after a shorter last chunk nothing follows
            have = zc1;
#pragma unroll
            for (int r = 0; r < NR; r++) {
                ba[r] += pk[r] >> PK_A;
                sm.bv[w][r][lane] += pk[r] & ((1u << PK_F) - 1u);
                sm.bf[w][r][lane] += (pk[r] >> PK_F) & ((1u << (PK_A - PK_F)) - 1u);
            }
        }
    }
    __syncwarp();
}

// Cell rows per warp tile of the compaction.  One row (two sample rows per
// plane) keeps the walk at 64 registers, 4 CTAs per SM, with 8 planes in flight
// per warp; at 1024^3 Float32: 0.675 ms, against 0.73 with 4 planes, 0.79 with
// 2 rows at 3 CTAs per SM and 1.00 with the classify tile's 4 rows at 2.
constexpr int CR = 1;
#ifndef COMPACT_MIN_CTAS
#define COMPACT_MIN_CTAS 4
#endif

template <class T>
__global__ void __launch_bounds__(256, COMPACT_MIN_CTAS) k_compact_mc(const Plan p, int nitems) {
    __shared__ CompactSmem sm;
    load_tables_mc_packed(sm.pk, sm.cs);
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int tiles_y = (p.cy + CR - 1) / CR;
    const int ntx = p.ntx > 0 ? p.ntx : p.tiles_x;  // x tiles tx0 .. tx0 + ntx - 1
    // persistent warps: take (y tile, x tile, segment) items in order from a counter
    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nitems) break;
        const int ty = item % tiles_y;
        const int tx = p.tx0 + (item / tiles_y) % ntx;
        const int seg = item / (tiles_y * ntx);
        compact_tile<T, CR>(p, sm, w, lane, tx, ty, seg, 0);
    }
}

// Batch: the work items of k_classify_batch, in the same order, each split
// into its WY / CR tiles of CR cell rows.
template <class T>
__global__ void __launch_bounds__(256, COMPACT_MIN_CTAS) k_compact_batch(const Plan p) {
    static_assert(WY % CR == 0, "compaction tiles split the classify tile");
    constexpr int SUB = WY / CR;
    __shared__ CompactSmem sm;
    load_tables_mc_packed(sm.pk, sm.cs);
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (;;) {
        unsigned item = 0;  // p.nitems * SUB < 2^31 (checked when the batch is planned)
        if (lane == 0) item = atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if ((int64_t)(item / SUB) >= p.nitems) break;
        const uint32_t v = p.item_vol[item / SUB];
        const BatchVol b = p.bvols[v];
        const int64_t local = (int64_t)(item / SUB) - b.item0;
        const int ty = (int)(local % b.tiles_y);
        const int tx = (int)((local / b.tiles_y) % b.tiles_x);
        const int seg = (int)(local / ((int64_t)b.tiles_y * b.tiles_x));
        compact_tile<T, CR>(vol_view(p, b), sm, w, lane, tx, ty * SUB + (int)(item % SUB), seg, v);
    }
}

// Resident CTAs of the compaction and the expansion on the current device, per
// instantiation, looked up once per device (devices of different models differ).
template <class T, class Q, class P> void list_grids(int *grid_a, int *grid_b) {
    constexpr int MAXDEV = 64;
    static std::mutex mu;
    static int ga[MAXDEV], gb[MAXDEV];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= MAXDEV) dev = 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!ga[dev]) {
        ga[dev] = resident_ctas((const void *)k_compact_mc<T>, 32 * WARPS);
        gb[dev] = expand_ctas((const void *)k_expand_mc<T, Q, P, EXP_ORDERED>);
    }
    *grid_a = ga[dev];
    *grid_b = gb[dev];
}

template <class T, class Q, class P> cudaError_t go(const Plan &p, int stage, cudaStream_t s) {
    int grid_a = 0, grid_b = 0;
    list_grids<T, Q, P>(&grid_a, &grid_b);
    if (stage == 0) {
        const int nitems = (p.ntx > 0 ? p.ntx : p.tiles_x) * ((p.cy + CR - 1) / CR) * p.nseg;
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
                                            (p.nitems * (WY / CR) + WARPS - 1) / WARPS);
    cudaError_t e = cudaMemsetAsync(p.work, 0, sizeof(unsigned), s);
    if (e != cudaSuccess || grid < 1) return e;
    k_compact_batch<T><<<grid, 32 * WARPS, 0, s>>>(p);
    return cudaGetLastError();
}

template <class T, class Q, class P> cudaError_t expand_batch_t(const Plan &p, cudaStream_t s) {
    // per instantiation: resident CTAs on this device (thread-safe one-time initialisation)
    static const int grid = expand_ctas((const void *)k_expand_mc<T, Q, P, EXP_BATCH>);
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
    case MESH_DT_F16: return compact_batch_t<h16>(p, ctas, s);
    case MESH_DT_I16: return compact_batch_t<int16_t>(p, ctas, s);
    case MESH_DT_I8: return compact_batch_t<int8_t>(p, ctas, s);
    case MESH_DT_U8: return compact_batch_t<uint8_t>(p, ctas, s);
    case MESH_DT_F32: return compact_batch_t<float>(p, ctas, s);
    case MESH_DT_I32: return compact_batch_t<int32_t>(p, ctas, s);
    case MESH_DT_I64: return compact_batch_t<int64_t>(p, ctas, s);
    default: return compact_batch_t<double>(p, ctas, s);
    }
}

cudaError_t launch_expand_batch(const Plan &p, int Q64, int P64, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return expand_batch_tt<uint16_t>(p, Q64, P64, s);
    case MESH_DT_F16: return expand_batch_tt<h16>(p, Q64, P64, s);
    case MESH_DT_I16: return expand_batch_tt<int16_t>(p, Q64, P64, s);
    case MESH_DT_I8: return expand_batch_tt<int8_t>(p, Q64, P64, s);
    case MESH_DT_U8: return expand_batch_tt<uint8_t>(p, Q64, P64, s);
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
    case MESH_DT_F16: return go_t<h16>(p, Q64, P64, stage, s);
    case MESH_DT_I16: return go_t<int16_t>(p, Q64, P64, stage, s);
    case MESH_DT_I8: return go_t<int8_t>(p, Q64, P64, stage, s);
    case MESH_DT_U8: return go_t<uint8_t>(p, Q64, P64, stage, s);
    case MESH_DT_F32: return go_t<float>(p, Q64, P64, stage, s);
    case MESH_DT_I32: return go_t<int32_t>(p, Q64, P64, stage, s);
    case MESH_DT_I64: return go_t<int64_t>(p, Q64, P64, stage, s);
    default: return go<double, double, double>(p, stage, s);
    }
}

}  // namespace mesh
