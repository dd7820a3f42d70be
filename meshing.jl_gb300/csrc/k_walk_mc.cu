// Marching Cubes in one walk over the volume.
//
// Replaces the cell loop of isosurface(sdf, ::MarchingCubes, X, Y, Z)
// (src/marching_cubes.jl:40-56) together with process_mc_voxel!
// (src/marching_cubes.jl:67-92).
//
// k_walk_mc classifies like K1 (k_classify.cu): a warp owns 31 x-cells by WY
// y-cells and walks one z segment, lane l loading sample x0+l of WY+1 rows
// per plane, one ballot per row giving the `v < iso` bits of the whole row.
// In the same walk every active cell is appended to a staging list: packed
// (x, y, z), case, its 8 corner values, and the vertex / face counts that
// precede it inside its piece (column x, y of the segment, in z order), which
// the walking lane holds in registers.  A warp takes STG_BLK slots at a time
// from one counter and fills them in the order it finds the cells; an entry
// may continue into the next block, and the unused end of the warp's last
// block gets case 0.  The per-piece totals go to the scan as from K1.
//
// After the scan, k_expand_mc<..., EXP_STAGED> (mesh_mc.cuh) writes each entry's
// vertices and faces at base(piece) + rank.  The volume is read once; the
// list holds only the ~2% active cells.
//
// If the list is too short, the walk still completes the counts, keeps what
// fits, and reports ERR_STAGE; *stage_next then holds the exact number of
// slots a repeated walk takes (each warp's demand does not depend on timing).
#define MESH_TBL static __device__ const
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_mc.cuh"

#include <algorithm>

namespace mesh {

namespace {

constexpr int U = 2;  // z planes loaded ahead

template <class T>
__global__ void __launch_bounds__(256, 3) k_walk_mc(const Plan p) {
    __shared__ uint32_t s_tab[256];  // vertices | faces << 8 of each case
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        const uint64_t t = MC_CASE_VERTS[i];
        s_tab[i] = (uint32_t)((t >> 48) & 15u) | ((uint32_t)((t >> 52) & 7u) << 8);
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int ty = blockIdx.y * WARPS + (threadIdx.x >> 5);
    if (ty >= p.tiles_y) return;  // warp-uniform
    const int tx = blockIdx.x;
    const int seg = blockIdx.z;
    const int xs = tx * TILE_X + lane;
    const int y0 = ty * WY;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < TILE_X && xs < p.cx;
    const T *vol = (const T *)p.vol;
    const int64_t sxy = p.nx * p.ny;
    const unsigned long long cap = (unsigned long long)p.ent_cap;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));

    bool rowok[WY + 1];
    const T *rowp[WY + 1];
#pragma unroll
    for (int r = 0; r <= WY; r++) {
        rowok[r] = xs < p.nx && y0 + r < p.ny;
        rowp[r] = rowok[r] ? vol + xs + p.nx * (int64_t)(y0 + r) : vol;
    }
    uint32_t cv[WY], cf[WY], ca[WY];  // running vertex / face / cell counts of the lane's pieces
#pragma unroll
    for (int r = 0; r < WY; r++) cv[r] = cf[r] = ca[r] = 0;
    unsigned long long cur = 0, end = 0;  // the warp's free staging slots [cur, end)
    bool over = false;                    // an entry fell beyond the list
    const uint32_t xval = __ballot_sync(FULL, xs < p.nx);
    const uint32_t cellm = __ballot_sync(FULL, cellx);

    uint32_t mlo[WY + 1];
    T lov[WY + 1];  // samples of plane z
#pragma unroll
    for (int r = 0; r <= WY; r++) {
        lov[r] = rowok[r] ? ldv(rowp[r] + sxy * zbeg) : T(0);
        mlo[r] = __ballot_sync(FULL, rowok[r] && below(lov[r], p));
    }

    for (int z = zbeg; z < zend; z += U) {
        T v[U][WY + 1];
        const int64_t off = sxy * (int64_t)(z + 1);
        if (z + U <= zend) {
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int r = 0; r <= WY; r++) v[u][r] = rowok[r] ? ldv(rowp[r] + off + sxy * u) : T(0);
        } else {
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int r = 0; r <= WY; r++)
                    v[u][r] = (rowok[r] && z + 1 + u <= zend) ? ldv(rowp[r] + off + sxy * u) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int zc = z + u;
            if (zc >= zend) break;  // warp-uniform
            uint32_t mhi[WY + 1];
            uint32_t all1 = xval, any1 = 0;
#pragma unroll
            for (int r = 0; r <= WY; r++) {
                mhi[r] = __ballot_sync(FULL, rowok[r] && below(v[u][r], p));
                all1 &= mlo[r] & mhi[r];
                any1 |= mlo[r] | mhi[r];
            }
            // warp-uniform early out: every corner of every cell of this step on one side
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
                    // slots for this row's n entries: the rest of the block, then a new block
                    const unsigned n = __popc(actm);
                    const unsigned long long rem = end - cur;
                    unsigned long long nb = 0;
                    if (n > rem) {
                        if (lane == 0) nb = atomicAdd(p.stage_next, (unsigned long long)STG_BLK);
                        nb = __shfl_sync(FULL, nb, 0);
                    }
                    if ((actm >> lane) & 1u) {
                        const unsigned a = (mlo[r] >> lane) & 3u, b = (mlo[r + 1] >> lane) & 3u;
                        const unsigned c = (mhi[r] >> lane) & 3u, d = (mhi[r + 1] >> lane) & 3u;
                        const unsigned cm = (a & 1u) | ((a >> 1) << 1) | ((b >> 1) << 2) | ((b & 1u) << 3) |
                                            ((c & 1u) << 4) | ((c >> 1) << 5) | ((d >> 1) << 6) | ((d & 1u) << 7);
                        const unsigned k = __popc(actm & lt);
                        const unsigned long long e = k < rem ? cur + k : nb + (k - rem);
                        if (e < cap) {
                            p.ent_pos[e] = (unsigned long long)xs | ((unsigned long long)(y0 + r) << POS_BITS) |
                                           ((unsigned long long)zc << (2 * POS_BITS));
                            p.ent_cs[e] = (uint8_t)cm;
                            const T vals[8] = {a0, a1, b1, b0, c0, c1, d1, d0};
                            store8<T>((T *)p.ent_val + 8 * e, vals);
                            p.ent_rank[e] = make_uint2(cv[r], cf[r]);
                        } else {
                            over = true;
                        }
                        const uint32_t t = s_tab[cm];
                        cv[r] += t & 15u;
                        cf[r] += t >> 8;
                        ca[r] += 1;
                    }
                    if (n > rem) {
                        cur = nb + (n - rem);
                        end = nb + STG_BLK;
                    } else {
                        cur += n;
                    }
                }
            }
#pragma unroll
            for (int r = 0; r <= WY; r++) mlo[r] = mhi[r];
        }
#pragma unroll
        for (int r = 0; r <= WY; r++) lov[r] = v[U - 1][r];
    }
    // the unused end of the last block: case 0, no output
    for (unsigned long long e = cur + lane; e < end; e += 32)
        if (e < cap) p.ent_cs[e] = 0;
    if (__any_sync(FULL, over) && lane == 0) atomicOr(p.err, ERR_STAGE);

    if (cellx) {
        const int64_t np = p.pstride;
#pragma unroll
        for (int r = 0; r < WY; r++) {
            if (y0 + r < p.cy) {
                const int64_t i = piece(p, seg, y0 + r, xs);
                p.cnt[i] = cv[r];
                p.cnt[np + i] = cf[r];
                p.cnt[2 * np + i] = ca[r];
            }
        }
    }
}

template <class T> cudaError_t walk_t(const Plan &p, cudaStream_t s) {
    dim3 grid(p.tiles_x, (p.tiles_y + WARPS - 1) / WARPS, p.nseg);
    k_walk_mc<T><<<grid, 32 * WARPS, 0, s>>>(p);
    return cudaGetLastError();
}

template <class T, class Q, class P> cudaError_t expand_t(const Plan &p, cudaStream_t s) {
    // per instantiation: resident CTAs on this device (thread-safe one-time initialisation)
    static const int grid = expand_ctas((const void *)k_expand_mc<T, Q, P, EXP_STAGED>);
    k_expand_mc<T, Q, P, EXP_STAGED><<<grid, XW, 0, s>>>(p);
    return cudaGetLastError();
}

template <class T> cudaError_t expand_tt(const Plan &p, int Q64, int P64, cudaStream_t s) {
    if (Q64) return expand_t<T, double, double>(p, s);
    if (P64) return expand_t<T, float, double>(p, s);
    return expand_t<T, float, float>(p, s);
}

}  // namespace

cudaError_t launch_walk_mc(const Plan &p, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return walk_t<uint16_t>(p, s);
    case MESH_DT_F16: return walk_t<h16>(p, s);
    case MESH_DT_I16: return walk_t<int16_t>(p, s);
    case MESH_DT_I8: return walk_t<int8_t>(p, s);
    case MESH_DT_U8: return walk_t<uint8_t>(p, s);
    case MESH_DT_F32: return walk_t<float>(p, s);
    case MESH_DT_I32: return walk_t<int32_t>(p, s);
    case MESH_DT_I64: return walk_t<int64_t>(p, s);
    default: return walk_t<double>(p, s);
    }
}

cudaError_t launch_expand_staged_mc(const Plan &p, int Q64, int P64, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return expand_tt<uint16_t>(p, Q64, P64, s);
    case MESH_DT_F16: return expand_tt<h16>(p, Q64, P64, s);
    case MESH_DT_I16: return expand_tt<int16_t>(p, Q64, P64, s);
    case MESH_DT_I8: return expand_tt<int8_t>(p, Q64, P64, s);
    case MESH_DT_U8: return expand_tt<uint8_t>(p, Q64, P64, s);
    case MESH_DT_F32: return expand_tt<float>(p, Q64, P64, s);
    case MESH_DT_I32: return expand_tt<int32_t>(p, Q64, P64, s);
    case MESH_DT_I64: return expand_tt<int64_t>(p, Q64, P64, s);
    default: return expand_t<double, double, double>(p, s);
    }
}

}  // namespace mesh
