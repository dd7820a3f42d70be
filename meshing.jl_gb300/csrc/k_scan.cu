// K2 -- scan: exclusive prefix of the per-piece counts in the reference's
// emission order.
//
// The reference numbers vertices and faces by `push!` order, i.e. cells in
// lexicographic (x, y, z) order with z fastest (src/marching_cubes.jl:40,
// src/marching_tetrahedra.jl:144).  A piece (x, y, seg) is a z segment of one
// column, so the emission order of pieces is (x, y, seg) lexicographic, while
// the counts sit in memory as [seg][y][x] (x fastest, written coalesced by
// the classify kernel).
//
// Single volume (k_scan_reduce, k_scan_cols, k_scan_colsum, k_scan_down): the
// (y, seg) sequence of every column is cut into C runs; a warp takes one run of
// 32 columns (lane = x, so every access stays coalesced) and sums it; a warp
// per column scans its run sums, three CTAs scan the column sums (x order),
// and the warps walk their runs again writing the offsets.  No wait between
// CTAs.
//
// Batch of small volumes (k_scan_batch_vol): one CTA per volume, chained over
// the volumes (below).
//
// Batch (k_scan_batch): one CTA scans 32 columns of one volume: its warps
// split the (y, seg) sequence of every column, reduce, scan across warps
// through shared memory (one warp per counter: vertices, faces, active cells),
// scan the 32 column totals with warp shuffles, and chain the groups of 32
// columns of all volumes with a single-pass decoupled look-back (groups are
// taken in ticket order, so every predecessor is already resident).
// Look-back waits are bounded: on expiry the kernel sets ERR_SCAN_TIMEOUT in
// the device error word and finishes without hanging.
#include "mesh_internal.cuh"

#include <algorithm>

namespace mesh {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned long long FLAG_AGG = 1ull << 62;
constexpr unsigned long long FLAG_INC = 2ull << 62;
constexpr unsigned long long VAL_MASK = (1ull << 62) - 1;

__device__ __forceinline__ void st_release(unsigned long long *a, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(a), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *a) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
    return v;
}

// Exclusive prefix of tile `tile` for one counter, given its aggregate.
__device__ int64_t look_back(unsigned long long *state, int tile, int64_t agg, int spin_limit, unsigned *err) {
    if (tile == 0) {
        st_release(&state[0], FLAG_INC | (unsigned long long)agg);
        return 0;
    }
    st_release(&state[tile], FLAG_AGG | (unsigned long long)agg);
    int64_t excl = 0;
    int k = tile - 1;
    int spins = 0;
    while (k >= 0) {
        const unsigned long long w = ld_acquire(&state[k]);
        const unsigned long long f = w & ~VAL_MASK;
        if (f == 0) {
            if (++spins > spin_limit) {
                atomicOr(err, ERR_SCAN_TIMEOUT);
                break;
            }
            __nanosleep(64);
            continue;
        }
        excl += (int64_t)(w & VAL_MASK);
        if (f == FLAG_INC) break;
        k--;
    }
    st_release(&state[tile], FLAG_INC | (unsigned long long)(excl + agg));
    return excl;
}

// Scan tile `xt` of the (view) plan p -- columns 32*xt .. 32*xt+31 -- which is
// tile `gt` of `ntiles` in the look-back chain.  The CTA's nw warps split the
// (y, seg) sequence of every column.
__device__ __forceinline__ void scan_body(const Plan &p, int xt, int gt, int ntiles, int64_t (*s_part)[32][33],
                                          int64_t (*s_xpre)[32]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int x = xt * 32 + lane;
    const bool xok = x < p.cx;
    const int64_t L = (int64_t)p.cy * p.nseg;
    const int64_t per = (L + nw - 1) / nw;
    const int64_t j0 = min(L, (int64_t)w * per), j1 = min(L, j0 + per);
    const int64_t np = p.pstride;

    // piece index of emission step j of column x: (seg, y) advance seg fastest
    const int64_t dseg = (int64_t)p.cy * p.cx, wrap = (int64_t)p.cx - (int64_t)(p.nseg - 1) * dseg;
    auto first = [&](int &seg) {
        seg = (int)(j0 % p.nseg);
        return piece(p, seg, (int)(j0 / p.nseg), x);
    };
    auto next = [&](int64_t &i, int &seg) {
        if (++seg == p.nseg) {
            seg = 0;
            i += wrap;
        } else {
            i += dseg;
        }
    };
    constexpr int UN = 4;  // steps whose loads are issued together

    int64_t sum[NCNT];
#pragma unroll
    for (int c = 0; c < NCNT; c++) sum[c] = 0;
    if (xok) {
        int seg;
        int64_t i = first(seg), j = j0;
        for (; j + UN <= j1; j += UN) {
            int64_t ii[UN];
#pragma unroll
            for (int k = 0; k < UN; k++) {
                ii[k] = i;
                next(i, seg);
            }
#pragma unroll
            for (int c = 0; c < NCNT; c++)
#pragma unroll
                for (int k = 0; k < UN; k++) sum[c] += p.cnt[c * np + ii[k]];
        }
        for (; j < j1; j++) {
#pragma unroll
            for (int c = 0; c < NCNT; c++) sum[c] += p.cnt[c * np + i];
            next(i, seg);
        }
    }
#pragma unroll
    for (int c = 0; c < NCNT; c++) s_part[c][w][lane] = sum[c];
    __syncthreads();

    if (w < NCNT) {  // warp c scans counter c
        const int c = w;
        int64_t tot = 0;  // column total; s_part becomes the per-warp exclusive prefix
        for (int k = 0; k < nw; k++) {
            const int64_t a = s_part[c][k][lane];
            s_part[c][k][lane] = tot;
            tot += a;
        }
        int64_t inc = tot;  // inclusive scan across the 32 columns
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t a = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += a;
        }
        const int64_t agg = __shfl_sync(FULL, inc, 31);
        int64_t pre = 0;
        if (lane == 0) {
            pre = look_back(p.scan_state + (int64_t)c * ntiles, gt, agg, p.scan_spin_limit, p.err);
            if (gt == ntiles - 1) p.totals[c] = pre + agg;
        }
        pre = __shfl_sync(FULL, pre, 0);
        s_xpre[c][lane] = pre + inc - tot;
    }
    __syncthreads();

    if (xok) {
        int64_t b[NCNT];
#pragma unroll
        for (int c = 0; c < NCNT; c++) b[c] = s_xpre[c][lane] + s_part[c][w][lane];
        int seg;
        int64_t i = first(seg), j = j0;
        for (; j + UN <= j1; j += UN) {
            int64_t ii[UN];
            uint32_t v[NCNT][UN];
#pragma unroll
            for (int k = 0; k < UN; k++) {
                ii[k] = i;
                next(i, seg);
            }
#pragma unroll
            for (int c = 0; c < NCNT; c++)
#pragma unroll
                for (int k = 0; k < UN; k++) v[c][k] = p.cnt[c * np + ii[k]];
#pragma unroll
            for (int k = 0; k < UN; k++)
#pragma unroll
                for (int c = 0; c < NCNT; c++) {
                    p.base[c * np + ii[k]] = b[c];
                    b[c] += v[c][k];
                }
        }
        for (; j < j1; j++) {
#pragma unroll
            for (int c = 0; c < NCNT; c++) {
                p.base[c * np + i] = b[c];
                b[c] += p.cnt[c * np + i];
            }
            next(i, seg);
        }
    }
}

// ---- single volume: reduce, scan of the run sums, downsweep ----

// Runs per column and steps per run for a plan: at most 128 runs (the column
// scan takes 4 rounds of 32) of at least 16 steps, and at most 2^20 run sums
// per counter.
struct ScanGeom {
    int G, C;     // column groups of 32, runs per column
    int64_t per;  // (y, seg) steps per run
};
inline ScanGeom scan_geom(const Plan &p) {
    ScanGeom g;
    g.G = (p.cx + 31) / 32;
    const int64_t L = (int64_t)p.cy * p.nseg;
    int64_t C = std::min<int64_t>(128, std::max<int64_t>(1, L / 16));
    C = std::min<int64_t>(C, std::max<int64_t>(1, ((int64_t)1 << 20) / (32 * (int64_t)g.G)));
    g.C = (int)std::max<int64_t>(1, C);
    g.per = (L + g.C - 1) / g.C;
    return g;
}

// Piece index of step j of column x: (seg, y) with seg fastest.
struct ColWalk {
    int64_t i;
    int seg;
    __device__ ColWalk(const Plan &p, int64_t j, int x) {
        seg = (int)(j % p.nseg);
        i = piece(p, seg, (int)(j / p.nseg), x);
    }
    __device__ void next(const Plan &p) {
        if (++seg == p.nseg) {
            seg = 0;
            i += (int64_t)p.cx - (int64_t)(p.nseg - 1) * p.cy * p.cx;
        } else {
            i += (int64_t)p.cy * p.cx;
        }
    }
};

// part[k][x][c]: sum of counter k over run c of column x (x < 32 G; columns past
// cx sum to 0).
__global__ void __launch_bounds__(256) k_scan_reduce(const Plan p, int G, int C, int64_t per) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int c = blockIdx.y * 8 + w;
    if (c >= C) return;  // warp-uniform
    const int x = blockIdx.x * 32 + lane;
    const int64_t L = (int64_t)p.cy * p.nseg;
    const int64_t j0 = min(L, (int64_t)c * per), j1 = min(L, j0 + per);
    const int64_t np = p.pstride;
    int64_t sum[NCNT] = {0, 0, 0};
    static_assert(NCNT == 3, "three counters");
    if (x < p.cx) {
        ColWalk cw(p, j0, x);
        int64_t j = j0;
        constexpr int UN = 4;
        for (; j + UN <= j1; j += UN) {
            int64_t ii[UN];
#pragma unroll
            for (int k = 0; k < UN; k++) {
                ii[k] = cw.i;
                cw.next(p);
            }
#pragma unroll
            for (int k = 0; k < NCNT; k++)
#pragma unroll
                for (int u = 0; u < UN; u++) sum[k] += p.cnt[k * np + ii[u]];
        }
        for (; j < j1; j++) {
#pragma unroll
            for (int k = 0; k < NCNT; k++) sum[k] += p.cnt[k * np + cw.i];
            cw.next(p);
        }
    }
    long long *part = (long long *)p.scan_state;
    const int64_t E = (int64_t)32 * G * C;
#pragma unroll
    for (int k = 0; k < NCNT; k++) part[k * E + (int64_t)x * C + c] = sum[k];
}

// Per column (a warp per counter and column): the run sums become exclusive
// prefixes inside the column, and the column's total goes to col[k][x].
__global__ void __launch_bounds__(256) k_scan_cols(const Plan p, int G, int C) {
    const int lane = threadIdx.x & 31;
    const int64_t ncol = (int64_t)32 * G;
    const int64_t wid = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (wid >= NCNT * ncol) return;  // warp-uniform
    const int k = (int)(wid / ncol);
    const int64_t x = wid % ncol;
    long long *r = (long long *)p.scan_state + (k * ncol + x) * C;
    long long *col = (long long *)p.scan_state + (int64_t)NCNT * ncol * C;
    long long carry = 0;
    for (int c0 = 0; c0 < C; c0 += 32) {  // C <= 128: at most 4 rounds
        const int c = c0 + lane;
        const long long v = c < C ? r[c] : 0;
        long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += u;
        }
        if (c < C) r[c] = carry + inc - v;
        carry += __shfl_sync(FULL, inc, 31);
    }
    if (lane == 0) col[k * ncol + x] = carry;
}

// In place: col[k][x] becomes the exclusive prefix of column x; totals[k] the
// sum of all.  CTA k scans counter k; a thread owns a contiguous range of columns.
__global__ void __launch_bounds__(1024) k_scan_colsum(const Plan p, int G, int C) {
    __shared__ long long s_w[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int k = blockIdx.x;
    const int64_t ncol = (int64_t)32 * G;
    long long *a = (long long *)p.scan_state + (int64_t)NCNT * ncol * C + k * ncol;
    const int64_t q = (ncol + 1023) / 1024;
    const int64_t x0 = min(ncol, (int64_t)tid * q), x1 = min(ncol, x0 + q);
    long long sum = 0;
    for (int64_t x = x0; x < x1; x++) sum += a[x];
    long long inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) s_w[w] = inc;
    __syncthreads();
    if (w == 0) {
        const long long v = s_w[lane];
        long long vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(FULL, vi, o);
            if (lane >= o) vi += u;
        }
        s_w[lane] = vi - v;  // exclusive prefix of warp `lane`
        if (lane == 31) p.totals[k] = vi;
    }
    __syncthreads();
    long long run = s_w[w] + inc - sum;
    for (int64_t x = x0; x < x1; x++) {
        const long long v = a[x];
        a[x] = run;
        run += v;
    }
}

// Each warp walks its run again, writing base[k] of every piece.
__global__ void __launch_bounds__(256) k_scan_down(const Plan p, int G, int C, int64_t per) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int c = blockIdx.y * 8 + w;
    if (c >= C) return;  // warp-uniform
    const int x = blockIdx.x * 32 + lane;
    if (x >= p.cx) return;
    const int64_t L = (int64_t)p.cy * p.nseg;
    const int64_t j0 = min(L, (int64_t)c * per), j1 = min(L, j0 + per);
    const int64_t np = p.pstride;
    const long long *part = (const long long *)p.scan_state;
    const int64_t ncol = (int64_t)32 * G, E = ncol * C;
    const long long *col = part + NCNT * E;
    int64_t b[NCNT];
#pragma unroll
    for (int k = 0; k < NCNT; k++) b[k] = col[k * ncol + x] + part[k * E + (int64_t)x * C + c];
    ColWalk cw(p, j0, x);
    int64_t j = j0;
    constexpr int UN = 4;
    for (; j + UN <= j1; j += UN) {
        int64_t ii[UN];
        uint32_t v[NCNT][UN];
#pragma unroll
        for (int u = 0; u < UN; u++) {
            ii[u] = cw.i;
            cw.next(p);
        }
#pragma unroll
        for (int k = 0; k < NCNT; k++)
#pragma unroll
            for (int u = 0; u < UN; u++) v[k][u] = p.cnt[k * np + ii[u]];
#pragma unroll
        for (int u = 0; u < UN; u++)
#pragma unroll
            for (int k = 0; k < NCNT; k++) {
                p.base[k * np + ii[u]] = b[k];
                b[k] += v[k][u];
            }
    }
    for (; j < j1; j++) {
#pragma unroll
        for (int k = 0; k < NCNT; k++) {
            p.base[k * np + cw.i] = b[k];
            b[k] += p.cnt[k * np + cw.i];
        }
        cw.next(p);
    }
}

// Batch: the scan tiles of all volumes, volumes in order, form one look-back
// chain, so every piece gets its offset in the batch's concatenated output and
// a volume's first piece gives the volume's first vertex and face.
__global__ void __launch_bounds__(1024) k_scan_batch(const Plan p) {
    __shared__ int s_tile;
    __shared__ int64_t s_part[NCNT][32][33];
    __shared__ int64_t s_xpre[NCNT][32];
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(p.scan_ticket, 1u);
    __syncthreads();
    const int t = s_tile;
    const BatchVol b = p.bvols[p.stile_vol[t]];
    scan_body(vol_view(p, b), t - b.stile0, t, p.nstiles, s_part, s_xpre);
}

// Batch of small volumes (every volume at most a few 32-column groups wide),
// one CTA per volume in ticket order: the volume's groups are reduced to its
// totals, one decoupled look-back over the volumes gives its offset, and the
// groups are scanned again in x order from that offset (the second read of the
// counts mostly hits the caches).  A chain of volumes instead of groups, and a
// CTA's fixed costs paid once per volume.
__global__ void __launch_bounds__(1024) k_scan_batch_vol(const Plan p) {
    __shared__ int s_v;
    __shared__ int64_t s_part[NCNT][32][33];
    __shared__ int64_t s_xpre[NCNT][32];
    __shared__ int64_t s_run[NCNT];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) s_v = (int)atomicAdd(p.scan_ticket, 1u);
    if (threadIdx.x < NCNT) s_run[threadIdx.x] = 0;
    __syncthreads();
    const int v = s_v;
    const BatchVol bv = p.bvols[v];
    const Plan q = vol_view(p, bv);
    const int T = bv.cx ? (bv.cx + 31) / 32 : 0;
    const int64_t L = (int64_t)q.cy * q.nseg;
    const int64_t per = (L + nw - 1) / nw;
    const int64_t j0 = min(L, (int64_t)w * per), j1 = min(L, j0 + per);
    const int64_t np = q.pstride;
    const int64_t dseg = (int64_t)q.cy * q.cx, wrap = (int64_t)q.cx - (int64_t)(q.nseg - 1) * dseg;
    // the lane's column sums over the warp's (y, seg) range in tile xt
    auto partial = [&](int xt, int64_t (&sum)[NCNT]) {
        const int x = xt * 32 + lane;
#pragma unroll
        for (int c = 0; c < NCNT; c++) sum[c] = 0;
        if (x >= q.cx) return;
        int seg = (int)(j0 % q.nseg);
        int64_t i = piece(q, seg, (int)(j0 / q.nseg), x);
        for (int64_t j = j0; j < j1; j++) {
#pragma unroll
            for (int c = 0; c < NCNT; c++) sum[c] += q.cnt[c * np + i];
            if (++seg == q.nseg) {
                seg = 0;
                i += wrap;
            } else {
                i += dseg;
            }
        }
    };
    // pass 1: the volume's totals
    int64_t acc[NCNT] = {0, 0, 0};
    for (int xt = 0; xt < T; xt++) {
        int64_t sum[NCNT];
        partial(xt, sum);
#pragma unroll
        for (int c = 0; c < NCNT; c++) acc[c] += sum[c];
    }
    // block reduce per counter
#pragma unroll
    for (int c = 0; c < NCNT; c++) {
        int64_t a = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(FULL, a, o);
        if (lane == 0) s_part[c][w][0] = a;
    }
    __syncthreads();
    if (w < NCNT) {
        const int c = w;
        int64_t a = lane < nw ? s_part[c][lane][0] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(FULL, a, o);
        if (lane == 0) {
            const int64_t pre = look_back(p.scan_state + (int64_t)c * p.nvols, v, a, p.scan_spin_limit, p.err);
            s_run[c] = pre;
            if (v == p.nvols - 1) p.totals[c] = pre + a;
        }
    }
    __syncthreads();
    // pass 2: every tile from the running offset
    for (int xt = 0; xt < T; xt++) {
        int64_t sum[NCNT];
        partial(xt, sum);
#pragma unroll
        for (int c = 0; c < NCNT; c++) s_part[c][w][lane] = sum[c];
        __syncthreads();
        if (w < NCNT) {
            const int c = w;
            int64_t tot = 0;
            for (int k = 0; k < nw; k++) {
                const int64_t a = s_part[c][k][lane];
                s_part[c][k][lane] = tot;
                tot += a;
            }
            int64_t inc = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t a = __shfl_up_sync(FULL, inc, o);
                if (lane >= o) inc += a;
            }
            s_xpre[c][lane] = s_run[c] + inc - tot;
            __syncwarp();
            if (lane == 31) s_run[c] += inc;
        }
        __syncthreads();
        const int x = xt * 32 + lane;
        if (x < q.cx) {
            int64_t b[NCNT];
#pragma unroll
            for (int c = 0; c < NCNT; c++) b[c] = s_xpre[c][lane] + s_part[c][w][lane];
            int seg = (int)(j0 % q.nseg);
            int64_t i = piece(q, seg, (int)(j0 / q.nseg), x);
            for (int64_t j = j0; j < j1; j++) {
#pragma unroll
                for (int c = 0; c < NCNT; c++) {
                    const uint32_t cv = q.cnt[c * np + i];
                    q.base[c * np + i] = b[c];
                    b[c] += cv;
                }
                if (++seg == q.nseg) {
                    seg = 0;
                    i += wrap;
                } else {
                    i += dseg;
                }
            }
        }
        __syncthreads();
    }
}

// First vertex / face of every volume: the scanned offset of its first piece
// in emission order (x = y = seg = 0).  A volume without cells shares the
// offset of the next piece, or the totals.
__global__ void k_batch_offsets(const Plan p) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v > p.nvols) return;
    int64_t ov = p.totals[0], of = p.totals[1];
    if (v < p.nvols) {
        const int64_t i = p.bvols[v].piece0;
        if (i < p.pstride) {
            ov = p.base[i];
            of = p.base[p.pstride + i];
        }
    }
    p.vol_off[2 * v] = ov;
    p.vol_off[2 * v + 1] = of;
}

}  // namespace

// Bytes of the scan scratch (scan_state) of a single-volume plan.
size_t scan_scratch_bytes(const Plan &p) {
    const ScanGeom g = scan_geom(p);
    return (size_t)NCNT * 32 * g.G * (g.C + 1) * sizeof(long long);  // run sums, column sums
}

cudaError_t launch_scan_batch(const Plan &p, int threads, cudaStream_t s, bool per_volume) {
    if (per_volume && p.nvols > 0) {
        cudaError_t e = cudaMemsetAsync(p.scan_state, 0, sizeof(unsigned long long) * NCNT * (size_t)p.nvols, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(p.scan_ticket, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess) return e;
        k_scan_batch_vol<<<p.nvols, threads, 0, s>>>(p);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        k_batch_offsets<<<(p.nvols + 1 + 255) / 256, 256, 0, s>>>(p);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(p.scan_state, 0, sizeof(unsigned long long) * NCNT * (size_t)p.nstiles, s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(p.scan_ticket, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    // no cells at all: the totals stay zero (cleared by the caller)
    if (p.nstiles > 0) k_scan_batch<<<p.nstiles, threads, 0, s>>>(p);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_batch_offsets<<<(p.nvols + 1 + 255) / 256, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_scan(const Plan &p, cudaStream_t s) {
    const ScanGeom g = scan_geom(p);
    const dim3 grid(g.G, (g.C + 7) / 8);
    k_scan_reduce<<<grid, 256, 0, s>>>(p, g.G, g.C, g.per);
    k_scan_cols<<<(int)((NCNT * 32 * (int64_t)g.G + 7) / 8), 256, 0, s>>>(p, g.G, g.C);
    k_scan_colsum<<<NCNT, 1024, 0, s>>>(p, g.G, g.C);
    k_scan_down<<<grid, 256, 0, s>>>(p, g.G, g.C, g.per);
    return cudaGetLastError();
}

// ---- a few prefix values for the host (the pipelined host path's split points) ----

namespace {
__global__ void k_gather(const int64_t *src, const GatherIdx g, int64_t *dst) {
    if ((int)threadIdx.x < g.n) dst[threadIdx.x] = src[g.idx[threadIdx.x]];
}
}  // namespace

cudaError_t launch_gather(const int64_t *src, const GatherIdx &g, int64_t *dst, cudaStream_t s) {
    if (g.n < 1 || g.n > GATHER_MAX) return cudaErrorInvalidValue;
    k_gather<<<1, GATHER_MAX, 0, s>>>(src, g, dst);
    return cudaGetLastError();
}

}  // namespace mesh
