// K3 (Marching Cubes), direct form -- the active cells' vertices and faces
// written straight from the volume at the scanned offsets, with no list of
// active cells in between.
//
// Replaces process_mc_voxel! (src/marching_cubes.jl:67-92), vertex_interp
// (:100-104) and mc_vert_points (:111-120) for single volumes.
//
// Work item: one warp tile of 31 x-cells by one cell row y, through one z
// segment; items are taken in (y, segment, x tile) order, so the write front
// of every column's output advances together and the sample row y + 1 an item
// shares with the next row's item is still in L2.  The classify kernel leaves,
// per (x tile, cell row, 8-plane chunk), a 32-bit mask of the columns with an
// active cell (cmask).  For each active chunk the warp
//   1. loads the chunk's 9 sample planes of rows y and y + 1, only in the
//      lanes whose sample an active cell uses (a lane whose cells are all on
//      one side reads nothing: about 6% of the volume's sectors at 1024^3),
//      and keeps them in the warp's shared memory;
//   2. classifies the 8 steps with one ballot per sample row and one lookup
//      of the case's packed word per cell (mesh_case.cuh);
//   3. numbers the active cells with one warp scan of a packed
//      (vertices | faces << 12 | cells << 23) word, and marks each cell's
//      first vertex and face task in two bitmaps;
//   4. maps all 32 lanes onto the chunk's vertex tasks, then its face tasks:
//      a task finds its cell from the bitmap word and a population count.
// The cells of one lane are consecutive in the emission order (x-major,
// z-fastest), so task t of lane l's cells goes to G[l] + t, G[l] being the
// lane's next global vertex (face) minus its first task.
#define MESH_TBL static __device__ const
#include "mesh_internal.cuh"
#include "mesh_tables.h"
#include "mesh_case.cuh"
#include "mesh_mc.cuh"

#include <algorithm>
#include <mutex>

namespace mesh {

namespace {

constexpr int DW = 8;                                          // warps per CTA
constexpr int NPL = ZC + 1;                                    // sample planes of a chunk
constexpr int MAXC = TILE_X * ZC;                              // cells of a chunk tile
constexpr int VBW = (MAXC * MC_MAX_VERTS + 31) / 32;           // vertex-task bitmap words
constexpr int FBW = (MAXC * MC_MAX_FACES + 31) / 32;           // face-task bitmap words
static_assert(MAXC * MC_MAX_VERTS < (1 << 12) && MAXC * MC_MAX_FACES < (1 << 11) && MAXC < (1 << 9),
              "a warp's chunk totals fit the packed scan word");
// Node table of a warp: x nodes x0 .. x0+31 at 0..31, y nodes y, y+1 at 32, 33,
// z nodes zc0 .. zc0+8 at 34..42; the spacing of a node is stored with it.
constexpr int NT = 44, NY = 32, NZ = 34;

// How positions are evaluated: P (the LinRange / quotient promotion) and the output.
//   PM_F32: P Float32, Float32 output:  fl32(p1 + fl32(mu * d))
//   PM_MIX: P Float64, Float32 output:  float pairs (fast_f32_pos) for a Float32
//           quotient, FP64 when undecided or for a Float64 quotient
//   PM_F64: Float64 output:             fl64(p1 + fl64(mu * d))
constexpr int PM_F32 = 0, PM_MIX = 1, PM_F64 = 2;

template <int PM> struct Nodes;
template <> struct Nodes<PM_F32> { float p[NT], d[NT]; };
template <> struct Nodes<PM_MIX> { float p[NT], pl[NT], d[NT], dl[NT]; };
template <> struct Nodes<PM_F64> { double p[NT], d[NT]; };

// Shared memory of one warp.
template <class T, int PM> struct DirectWarp {
    T val[NPL * 64];             // the chunk's samples: [plane][row y, y+1][lane]
    long long gv[32], gf[32];    // per lane: global vertex / face of task 0
    Nodes<PM> nd;
    uint32_t rec[MAXC];          // cell: case | lane << 8 | step << 13 | first vertex task << 16
    uint16_t fst[MAXC];          // the cell's first face task
    uint32_t vbm[VBW], fbm[FBW]; // bit t set: task t is a cell's first
};

// Per case and vertex slot: the edge's start / end corner as offsets into a
// warp's val array (dz*64 + dy*32 + dx) and its moving axis; per case and face
// slot: the three local vertex slots (4 bits each).
struct CaseTabs {
    uint16_t ev[256 * MC_MAX_VERTS];
    uint16_t ef[256 * MC_MAX_FACES];
    uint32_t pc[256];  // by walk index: packed counts (mesh_case.cuh), cube case in bits 24-31
};
template <class T, int PM> constexpr size_t direct_smem() {
    return (sizeof(CaseTabs) + 15) / 16 * 16 + DW * sizeof(DirectWarp<T, PM>);
}

__device__ __forceinline__ uint32_t lanemask_le(int lane) { return (2u << lane) - 1u; }
__device__ __forceinline__ int coff(int k) { return cdz(k) * 64 + cdy(k) * 32 + cdx(k); }

// Table entries of node i of one axis (global index gi of an axis of n nodes;
// tables of that axis at offset `ax0` of each table array).
template <int PM>
__device__ __forceinline__ void put_node(Nodes<PM> &nd, int i, const Tabs &tb, int64_t ax0, int64_t gi) {
    if (PM == PM_F32) {
        nd.p[i] = __ldg(tb.xpf + ax0 + gi);
        nd.d[i] = __ldg(tb.dxf + ax0 + gi);
    } else if (PM == PM_MIX) {
        Nodes<PM_MIX> &m = reinterpret_cast<Nodes<PM_MIX> &>(nd);
        m.p[i] = __ldg(tb.split + ax0 + gi);
        m.pl[i] = __ldg(tb.split + tb.ntab + ax0 + gi);
        m.d[i] = __ldg(tb.split + 2 * tb.ntab + ax0 + gi);
        m.dl[i] = __ldg(tb.split + 3 * tb.ntab + ax0 + gi);
    } else {
        Nodes<PM_F64> &m = reinterpret_cast<Nodes<PM_F64> &>(nd);
        m.p[i] = __ldg(tb.xp + ax0 + gi);
        m.d[i] = __ldg(tb.dx + ax0 + gi);
    }
}

// p1 + mu * (p1 - p1) on an axis the edge does not move along, when p1 == 0 or
// mu is not finite (otherwise it is p1): evaluated in P, rounded to the output.
template <class P, class O> __device__ __noinline__ O still_slow(double c, double mu) {
    return (O)Ar<P>::add((P)c, Ar<P>::mul((P)mu, P(0)));
}

// Vertex task: the crossing on the edge whose start / end corners sit at val
// offsets oa / ob of cell (lane ln, step s), moving along axis ax.
template <class T, class Q, class P, int PM>
__device__ __forceinline__ void direct_vertex(const Plan &p, const Tabs &tb, const DirectWarp<T, PM> &w, int ln,
                                              int s, int oa, int ob, int ax, int x, int y, int z, int64_t out) {
    const T va = w.val[s * 64 + ln + oa], vb = w.val[s * 64 + ln + ob];
    const Q mu = quotient<Q>(va, vb, p);
    const bool fin = isfinite(mu);
    // the start corner's nodes; the spacing of the moving axis is its lower node's
    const int xi = ln + (oa & 1), yi = NY + ((oa >> 5) & 1), zi = NZ + s + (oa >> 6);
    const int lo = ax == 0 ? ln : (ax == 1 ? NY : NZ + s);
    const int ni = ax == 0 ? xi : (ax == 1 ? yi : zi);
    const bool neg = ni != lo;
    if (PM == PM_F64) {
        const Nodes<PM_F64> &nd = reinterpret_cast<const Nodes<PM_F64> &>(w.nd);
        const P m = (P)mu;
        const double d = neg ? -nd.d[lo] : nd.d[lo];
        const double r = (double)Ar<P>::add((P)nd.p[ni], Ar<P>::mul(m, (P)d));
        double o0 = nd.p[xi], o1 = nd.p[yi], o2 = nd.p[zi];
        if (!fin || o0 == 0.0 || o1 == 0.0 || o2 == 0.0) {
            o0 = still_slow<P, double>(o0, (double)mu);
            o1 = still_slow<P, double>(o1, (double)mu);
            o2 = still_slow<P, double>(o2, (double)mu);
        }
        double *o = (double *)p.verts + 3 * out;
        o[0] = ax == 0 ? r : o0;
        o[1] = ax == 1 ? r : o1;
        o[2] = ax == 2 ? r : o2;
    } else {
        float r;
        if (PM == PM_F32) {
            const Nodes<PM_F32> &nd = reinterpret_cast<const Nodes<PM_F32> &>(w.nd);
            const float d = neg ? -nd.d[lo] : nd.d[lo];
            r = (float)Ar<P>::add((P)nd.p[ni], Ar<P>::mul((P)mu, (P)d));
        } else {
            const Nodes<PM_MIX> &nd = reinterpret_cast<const Nodes<PM_MIX> &>(w.nd);
            const float dh = nd.d[lo], dl = nd.dl[lo];
            // (a Float64 quotient -- Int / Int on integer data -- has no float-pair form)
            const bool done = sizeof(Q) == 4 && fin && !p.force_fp64 &&
                              fast_f32_pos((float)mu, nd.p[ni], nd.pl[ni], neg ? -dh : dh, neg ? -dl : dl, r);
            if (!done) {
                // the Float64 expression, from the double tables
                const int64_t ax0 = ax == 0 ? 0 : (ax == 1 ? tb.nx : tb.nx + tb.ny);
                const int64_t g = ax == 0 ? x : (ax == 1 ? y : z);  // the lower node
                const double dd = __ldg(tb.dx + ax0 + g);
                r = moving_fp64<P>(__ldg(tb.xp + ax0 + g + (neg ? 1 : 0)), neg ? -dd : dd, (double)mu);
            }
        }
        // p[] is the node rounded to float (PM_MIX: its high part)
        const Nodes<PM_F32> &nf = reinterpret_cast<const Nodes<PM_F32> &>(w.nd);
        float o0 = nf.p[xi], o1 = nf.p[yi], o2 = nf.p[zi];
        if (!fin || o0 == 0.0f || o1 == 0.0f || o2 == 0.0f) {
            if (PM == PM_MIX) {
                // the literal expression on the Float64 nodes (a node that rounds
                // to a float zero need not be zero)
                const F3 ov = still_fp64<P>(tb.xp, tb.yp, tb.zp, tb.xpf, tb.ypf, tb.zpf, x + (oa & 1),
                                            y + ((oa >> 5) & 1), z + (oa >> 6), (double)mu);
                o0 = ov.v[0];
                o1 = ov.v[1];
                o2 = ov.v[2];
            } else {
                o0 = still_slow<P, float>(o0, (double)mu);
                o1 = still_slow<P, float>(o1, (double)mu);
                o2 = still_slow<P, float>(o2, (double)mu);
            }
        }
        float *o = (float *)p.verts + 3 * out;
        o[0] = ax == 0 ? r : o0;
        o[1] = ax == 1 ? r : o1;
        o[2] = ax == 2 ? r : o2;
    }
}

template <class T, class Q, class P, int PM>
__device__ __forceinline__ void direct_tile(const Plan &p, const Tabs &tb, DirectWarp<T, PM> &w, const CaseTabs &ct,
                                            int lane, int tx, int y, int seg) {
    const int x0 = tx * TILE_X;
    const int xs = x0 + lane;
    const int zbeg = seg * p.zs;
    const int zend = min(zbeg + p.zs, p.cz);
    const bool cellx = lane < TILE_X && xs < p.cx;
    const bool have = xs < p.nx;
    const int64_t sxy = p.nx * p.ny;
    const T *row0 = (const T *)p.vol + (have ? xs : 0) + p.nx * (int64_t)y;
    const int64_t np = p.pstride;
    long long gv = 0, gf = 0;  // this lane's next global vertex / face
    if (cellx) {
        const int64_t i = piece(p, seg, y, xs);
        gv = p.base[i];
        gf = p.base[np + i];
    }
    // x and y nodes of the item
    if (have) put_node<PM>(w.nd, lane, tb, 0, xs);
    if (lane < 2) put_node<PM>(w.nd, NY + lane, tb, tb.nx, y + lane);
    const uint32_t cellm = __ballot_sync(FULL, cellx);
    const int nch = (zend - zbeg + ZC - 1) / ZC;
    const uint32_t *mrow = p.cmask + ((int64_t)tx * p.cy + y) * p.nchunks + (int64_t)seg * p.chunks_per_seg;
    for (int g = 0; 32 * g < nch; g++) {
        const uint32_t mine = 32 * g + lane < nch ? __ldg(mrow + 32 * g + lane) : 0u;
        uint32_t todo = __ballot_sync(FULL, mine != 0u);
        while (todo) {
            const int k = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint32_t m = __shfl_sync(FULL, mine, k) & cellm;
            if (m == 0u) continue;  // warp-uniform
            const int zc0 = zbeg + (32 * g + k) * ZC;
            const int ns = min(ZC, zend - zc0);  // z steps of this chunk
            // lane l's sample is used by cells l - 1 and l
            const bool ld = have && (((m | (m << 1)) >> lane) & 1u);
            T v[NPL][2];
            const T *a = row0 + sxy * (int64_t)zc0;
#pragma unroll
            for (int q = 0; q < NPL; q++) {
                const bool lq = ld && q <= ns;
                v[q][0] = lq ? ldv(a) : T(0);
                v[q][1] = lq ? ldv(a + p.nx) : T(0);
                a += sxy;
            }
            __syncwarp();  // the previous chunk's tasks are done with the node table
            if (lane < NPL && zc0 + lane < p.nz) put_node<PM>(w.nd, NZ + lane, tb, tb.nx + tb.ny, zc0 + lane);
            // per plane the lane's (x, x+1) sign fields of row y (bits 0-1) and
            // row y+1 (bits 4-5); a step's index is plane z | plane z+1 << 2
            uint32_t gq[NPL];
#pragma unroll
            for (int q = 0; q < NPL; q++) {
                const uint32_t m0 = __ballot_sync(FULL, below(v[q][0], p));
                const uint32_t m1 = __ballot_sync(FULL, below(v[q][1], p));
                gq[q] = ((m0 >> lane) & 3u) | (((m1 >> lane) << 4) & 0x30u);
                w.val[q * 64 + lane] = v[q][0];
                w.val[q * 64 + 32 + lane] = v[q][1];
            }
            const bool act = (m >> lane) & 1u;
            uint32_t pcs[ZC];
            uint32_t acc = 0;  // packed vertices | faces << 12 | cells << 23 of the lane's cells
#pragma unroll
            for (int s = 0; s < ZC; s++) {
                const uint32_t c = (act && s < ns) ? ct.pc[gq[s] | (gq[s + 1] << 2)] : 0u;
                pcs[s] = c;
                acc += c & 0xffffffu;
            }
            uint32_t inc = acc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(FULL, inc, o);
                if (lane >= o) inc += t;
            }
            const uint32_t tot = __shfl_sync(FULL, inc, 31);
            const uint32_t exc = inc - acc;
            const int VW = (int)(tot & 0xfffu), FW = (int)((tot >> 12) & 0x7ffu);
            uint32_t rv = exc & 0xfffu, rf = (exc >> 12) & 0x7ffu, rc = exc >> 23;
            w.gv[lane] = gv - (long long)rv;
            w.gf[lane] = gf - (long long)rf;
            gv += acc & 0xfffu;
            gf += (acc >> 12) & 0x7ffu;
            for (int i = lane; i < (VW + 31) / 32; i += 32) w.vbm[i] = 0u;
            for (int i = lane; i < (FW + 31) / 32; i += 32) w.fbm[i] = 0u;
            __syncwarp();
#pragma unroll
            for (int s = 0; s < ZC; s++) {
                const uint32_t c = pcs[s];
                if (c & 0xffffffu) {
                    w.rec[rc] = (c >> 24) | ((uint32_t)lane << 8) | ((uint32_t)s << 13) | (rv << 16);
                    w.fst[rc] = (uint16_t)rf;
                    atomicOr(&w.vbm[rv >> 5], 1u << (rv & 31));
                    atomicOr(&w.fbm[rf >> 5], 1u << (rf & 31));
                    rv += c & 0xfffu;
                    rf += (c >> 12) & 0x7ffu;
                    rc++;
                }
            }
            __syncwarp();
            // vertex tasks
            int cb = 0;
            for (int r = 0; 32 * r < VW; r++) {
                const uint32_t bits = w.vbm[r];
                const int t = 32 * r + lane;
                const int j = cb + __popc(bits & lanemask_le(lane)) - 1;
                cb += __popc(bits);
                if (t < VW) {
                    const uint32_t rec = w.rec[j];
                    const int cs = (int)(rec & 255u), ln = (int)((rec >> 8) & 31u), s = (int)((rec >> 13) & 7u);
                    const uint32_t ev = ct.ev[cs * MC_MAX_VERTS + (t - (int)(rec >> 16))];
                    const int oa = (int)(ev & 127u), ob = (int)((ev >> 7) & 127u), ax = (int)(ev >> 14);
                    const int64_t out = w.gv[ln] + t;
                    const int x = x0 + ln, z = zc0 + s;
                    if ((uint64_t)out < (uint64_t)p.verts_cap) {
                        direct_vertex<T, Q, P, PM>(p, tb, w, ln, s, oa, ob, ax, x, y, z, out);
                        if (p.vkey) {
                            // the edge's lower node; the cell owns the edge when, across
                            // each other axis, the edge lies on the cell's upper side or
                            // the cell is first
                            const int ox = ax == 0 ? 0 : (oa & 1), oy = ax == 1 ? 0 : ((oa >> 5) & 1),
                                      oz = ax == 2 ? 0 : (oa >> 6);
                            const bool own =
                                (ax == 0 || ox || x == 0) && (ax == 1 || oy || y == 0) && (ax == 2 || oz || z == 0);
                            const long long key =
                                ax + 3 * ((long long)(x + ox) + p.nx * ((long long)(y + oy) + p.ny * (long long)(z + oz)));
                            p.vkey[out] = key | (own ? (long long)(1ull << 63) : 0ll);
                        }
                    } else {
                        atomicOr(p.err, ERR_CAPACITY);
                    }
                }
            }
            // face tasks
            cb = 0;
            for (int r = 0; 32 * r < FW; r++) {
                const uint32_t bits = w.fbm[r];
                const int t = 32 * r + lane;
                const int j = cb + __popc(bits & lanemask_le(lane)) - 1;
                cb += __popc(bits);
                if (t < FW) {
                    const uint32_t rec = w.rec[j];
                    const int cs = (int)(rec & 255u), ln = (int)((rec >> 8) & 31u);
                    const unsigned sf = ct.ef[cs * MC_MAX_FACES + (t - (int)w.fst[j])];
                    const int64_t out = w.gf[ln] + t;
                    const long long vb1 = w.gv[ln] + (long long)(rec >> 16) + 1;  // 1-based
                    if ((uint64_t)out < (uint64_t)p.faces_cap) {
                        int64_t *o = p.faces + 3 * out;
                        o[0] = vb1 + (sf & 15u);
                        o[1] = vb1 + ((sf >> 4) & 15u);
                        o[2] = vb1 + ((sf >> 8) & 15u);
                    } else {
                        atomicOr(p.err, ERR_CAPACITY);
                    }
                }
            }
        }
    }
    __syncwarp();  // the next item rewrites the warp's node table
}

template <class T, class Q, class P, int PM>
// (at least 2 CTAs per SM: the Float32 paths take 72 registers and run 3 CTAs
// per SM, faster than the 64-register form at 4 CTAs: 1.08 against 1.11 ms at 1024^3)
__global__ void __launch_bounds__(32 * DW, 2) k_direct_mc(const Plan p, int nitems) {
    extern __shared__ __align__(16) unsigned char dsm[];
    CaseTabs &ct = *reinterpret_cast<CaseTabs *>(dsm);
    DirectWarp<T, PM> *sw = reinterpret_cast<DirectWarp<T, PM> *>(dsm + (sizeof(CaseTabs) + 15) / 16 * 16);
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        // packed count word (mesh_case.cuh) of walk index i, with the cube case in bits 24-31
        const unsigned cm = mc_case_of_index((unsigned)i);
        const uint64_t t = MC_CASE_VERTS[cm];
        ct.pc[i] = (uint32_t)((t >> 48) & 15u) | ((uint32_t)((t >> 52) & 7u) << PK_F) |
                   ((cm != 0u && cm != 255u) ? (1u << PK_A) : 0u) | (cm << 24);
        // vertex and face slots of cube case i
        const uint64_t tv = MC_CASE_VERTS[i], tf = MC_CASE_FACES[i];
        for (int k = 0; k < MC_MAX_VERTS; k++) {
            const int g = edge_info((int)((tv >> (4 * k)) & 15u));
            const int a = g & 7, b = (g >> 3) & 7, ax = (g >> 6) & 3;
            ct.ev[i * MC_MAX_VERTS + k] = (uint16_t)(coff(a) | (coff(b) << 7) | (ax << 14));
        }
        for (int k = 0; k < MC_MAX_FACES; k++) ct.ef[i * MC_MAX_FACES + k] = (uint16_t)((tf >> (12 * k)) & 0xfffu);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const Tabs tb = tabs_of(p);
    const int ntx = p.ntx > 0 ? p.ntx : p.tiles_x;  // x tiles tx0 .. tx0 + ntx - 1
    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(p.work, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= nitems) break;
        const int tx = p.tx0 + item % ntx;
        const int seg = (item / ntx) % p.nseg;
        const int y = item / (ntx * p.nseg);
        direct_tile<T, Q, P, PM>(p, tb, sw[wi], ct, lane, tx, y, seg);
    }
}

// Resident CTAs of k_direct_mc<T, Q, P, PM> on the current device, with its
// dynamic shared memory allowed (one-time per device and instantiation).
template <class T, class Q, class P, int PM> int direct_grid() {
    static std::mutex mu;
    static int grid[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!grid[dev]) {
        const void *fn = (const void *)k_direct_mc<T, Q, P, PM>;
        const int smem = (int)direct_smem<T, PM>();
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * DW, smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        cudaGetLastError();
        grid[dev] = per_sm * sms;
    }
    return grid[dev];
}

template <class T, class Q, class P, int PM> cudaError_t go(const Plan &p, cudaStream_t s) {
    const int grid = direct_grid<T, Q, P, PM>();
    const int nitems = (p.ntx > 0 ? p.ntx : p.tiles_x) * p.nseg * p.cy;
    if (grid < 1) return cudaErrorInvalidDevice;
    cudaError_t e = cudaMemsetAsync(p.work, 0, sizeof(unsigned), s);
    if (e != cudaSuccess || nitems < 1) return e;
    k_direct_mc<T, Q, P, PM><<<std::min(grid, (nitems + DW - 1) / DW), 32 * DW, direct_smem<T, PM>(), s>>>(p, nitems);
    return cudaGetLastError();
}

template <class T> cudaError_t go_t(const Plan &p, int Q64, int P64, cudaStream_t s) {
    if (p.out64) {
        if (Q64) return go<T, double, double, PM_F64>(p, s);
        return go<T, float, double, PM_F64>(p, s);
    }
    if (Q64) return go<T, double, double, PM_MIX>(p, s);  // integer data, Int iso, Float32 ranges
    if (P64) return go<T, float, double, PM_MIX>(p, s);
    return go<T, float, float, PM_F32>(p, s);
}

}  // namespace

// Direct Marching Cubes emission of a single volume (Plan::cmask from the
// classify walk, Plan::base from the scan); x tiles tx0 .. tx0 + ntx - 1 when
// ntx > 0.
cudaError_t launch_direct_mc(const Plan &p, int Q64, int P64, cudaStream_t s) {
    switch (p.T) {
    case MESH_DT_U16: return go_t<uint16_t>(p, Q64, P64, s);
    case MESH_DT_F16: return go_t<h16>(p, Q64, P64, s);
    case MESH_DT_I16: return go_t<int16_t>(p, Q64, P64, s);
    case MESH_DT_I8: return go_t<int8_t>(p, Q64, P64, s);
    case MESH_DT_U8: return go_t<uint8_t>(p, Q64, P64, s);
    case MESH_DT_F32: return go_t<float>(p, Q64, P64, s);
    case MESH_DT_I32: return go_t<int32_t>(p, Q64, P64, s);
    case MESH_DT_I64: return go_t<int64_t>(p, Q64, P64, s);
    default: return go<double, double, double, PM_F64>(p, s);
    }
}

}  // namespace mesh
